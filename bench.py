"""Benchmark: double-double GEMM throughput at n = 8192 on GB300.

Metric (the reference's headline): DD-GEMM GFLOP/s at
M = N = K = 8192 with the integer-exact tensor-core ("Ozaki") engine, next to
the plain FP64 error-free-transform engine on the same GPU, work counted as
2*M*N*K double-double flops.

A step is one C := alpha*A*B + beta*C at 8192^3 (alpha, beta random
double-double of magnitude 0.5..2, A/B/C with hi ~ U[-1,1), lo = hi*2^-53*U),
through the drop-in symbol a caller of the reference links (mgemm_64_), whose
automatic engine choice takes the tensor-core engine at this size.
  value : device-resident operands (1 GiB each, larger than L2), CUDA events
          around K steps on the library's stream, max over ranks.
  e2e   : the same call with pinned HOST buffers, so every step includes the
          host->device copies of A, B, C and the device->host copy of C;
          e2e_pageable: the same with ordinary (pageable) host arrays, as a
          Fortran or C caller hands them over.
Multi-GPU (torchrun): every rank runs its own independent GEMM (replicas; the
path needs no collective), value = total flops of all ranks / max time.

`--impl reference` times the reference's CPU implementation of the same
routine on this machine's host cores: the reference built from its own
sources where it is present (x86 development host), otherwise the C port of
its algorithm in oracle/ (the GPU machine), on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

METRIC = "DD-GEMM GFLOP/s n=8192, Ozaki-INT8 vs FP64-EFT, rel err <=1e-30; % roofline"
UNIT = "DD-GFLOP/s"
N_GEMM = 8192


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = float(s[2])
                for nm, v in zip(names, s[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def job_throughput(local_ms, work_per_rank, world, dist=None, device="cpu"):
    """Whole-job throughput of `world` independent replicas: each rank did
    `work_per_rank` units in `local_ms`; the job lasted as long as the slowest
    rank. Returns (units per second, max_ms)."""
    ms = float(local_ms)
    if dist is not None:
        import torch
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return world * work_per_rank / (ms * 1e-3), ms


def make_inputs(rng, n):
    mwb = ge._load("mwblas", os.path.join(ge.PKG, "mwblas.py"))
    A = mwb.dd_matrix(rng, n, n)
    B = mwb.dd_matrix(rng, n, n)
    C = mwb.dd_matrix(rng, n, n)

    def scal():
        mag = 0.5 + 1.5 * rng.random()
        s = mag if rng.random() < 0.5 else -mag
        return np.array([s, s * 2.0 ** -53 * (2 * rng.random() - 1)])
    return A, B, C, scal(), scal()


def run_ours(args, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    mwb = ge._load("mwblas", os.path.join(ge.PKG, "mwblas.py"))
    lib = mwb.MWBlas(os.path.join(ge.PKG, "libmwblas_gb300.so"))
    n = args.n
    rng = np.random.default_rng(1234 + rank)
    A, B, C0, alpha, beta = make_inputs(rng, n)
    dev = torch.device("cuda", local_rank)
    dA = torch.from_numpy(A).to(dev)
    dB = torch.from_numpy(B).to(dev)
    dC = torch.from_numpy(C0).to(dev)
    dC0 = dC.clone()
    stream = torch.cuda.current_stream(dev)
    lib.lib.mwblas_set_stream(stream.cuda_stream)

    lib.lib.mwblas_set_gemm_engine(0)   # AUTO: the drop-in call's own engine choice

    def step(engine=None, c=dC):
        lib.mgemm("N", "N", n, n, n, alpha, dA.data_ptr(), n, dB.data_ptr(), n, beta, c.data_ptr(), n, engine=engine)

    dist = None
    if world > 1:
        import torch.distributed as dist

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        dC.copy_(dC0)
        step()
    code, msg = lib.last_error()
    if code != 0:
        raise RuntimeError(f"mgemm_64_ failed: {code} {msg}")
    moduli = int(lib.lib.mwblas_last_ozaki_moduli())
    if moduli <= 0:
        raise RuntimeError("mgemm_64_ did not take the tensor-core engine")

    # ---- timed region: K steps, device-resident operands (each 1 GiB > L2).
    # The library records CUDA events around each engine phase on its stream,
    # which gives the residue-GEMM kernel's own duration per launch.
    l0 = lib.lib.mwblas_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lib.lib.mwblas_set_kernel_timing(1)
    phase = np.zeros(4)
    barrier()
    with ClockSampler(local_rank) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
            phase += [lib.lib.mwblas_last_phase_ms(i) for i in range(4)]
        ev1.record(stream)
        barrier()
    lib.lib.mwblas_set_kernel_timing(0)
    phase /= args.steps
    launches = lib.lib.mwblas_launch_count() - l0
    flops = 2.0 * n * n * n
    value, ms = job_throughput(ev0.elapsed_time(ev1) / args.steps, flops, world, dist, dev)
    value /= 1e9

    pk, pk_kind = peaks()

    # ---- e2e: pinned host buffers through the same C-ABI call
    hA = torch.from_numpy(A).pin_memory()
    hB = torch.from_numpy(B).pin_memory()
    hC = torch.from_numpy(C0).pin_memory()
    def host_calls(a_, b_, c_, calls):
        for _ in range(max(3, args.warmup)):   # warm-up calls, as for the device-timed steps
            lib.mgemm("N", "N", n, n, n, alpha, a_, n, b_, n, beta, c_, n)
        barrier()
        # each call timed on the host clock (the call returns with C back in host
        # memory); the median, as the host link is shared with other jobs
        per = []
        for _ in range(calls):
            t0 = time.perf_counter()
            lib.mgemm("N", "N", n, n, n, alpha, a_, n, b_, n, beta, c_, n)
            per.append((time.perf_counter() - t0) * 1e3)
        barrier()
        code_, msg_ = lib.last_error()
        if code_ != 0:
            raise RuntimeError(f"mgemm_64_ on host arrays failed: {code_} {msg_}")
        return per

    e_steps = max(1, min(args.steps, 5))
    per_call = host_calls(hA.data_ptr(), hB.data_ptr(), hC.data_ptr(), e_steps)
    e_val, e_ms = job_throughput(float(np.median(per_call)), flops, world, dist, dev)
    e2e = {"value": e_val / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": 3 * n * n * 16, "d2h_bytes_per_step": n * n * 16,
           "ms_per_step": e_ms, "stat": f"median of {e_steps} calls",
           "per_call_ms": [round(x, 2) for x in per_call], "api": "mgemm_64_ on pinned host arrays"}
    del hA, hB, hC
    # the same call on ordinary pageable numpy arrays
    pA, pB, pC = A.copy(), B.copy(), C0.copy()
    p_steps = max(1, min(args.steps, 3))
    per_call_p = host_calls(pA, pB, pC, p_steps)
    p_val, p_ms = job_throughput(float(np.median(per_call_p)), flops, world, dist, dev)
    e2e_pageable = {"value": p_val / 1e9, "unit": UNIT,
                    "h2d_bytes_per_step": 3 * n * n * 16, "d2h_bytes_per_step": n * n * 16,
                    "ms_per_step": p_ms, "stat": f"median of {p_steps} calls",
                    "per_call_ms": [round(x, 2) for x in per_call_p], "api": "mgemm_64_ on pageable host arrays"}
    del pA, pB, pC

    # ---- the plain FP64-EFT engine on the same GPU (one timed call)
    plain = None
    if not args.skip_plain:
        step(engine="plain", c=dC)   # warm
        barrier()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        step(engine="plain", c=dC)
        p1.record(stream)
        barrier()
        pms = p0.elapsed_time(p1)
        # FP64 lane operations per DD multiply-add and FP64-pipe activity, from the
        # ncu capture of the same kernel (sm__inst_executed_pipe_fp64 x 32 / MACs)
        prof = plain_profile()
        fp64_inst = n * n * n * prof.get("fp64_inst_per_mac", 7.5)
        plain = {"value": flops / (pms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": pms,
                 "kernel": "k_gemm_plain_tma (TMA-staged tiles, FP64 error-free transforms)",
                 "fp64_inst_per_s": fp64_inst / (pms * 1e-3), "fp64_inst_per_mac": prof.get("fp64_inst_per_mac"),
                 "fp64_pipe_active_pct_ncu": prof.get("fp64_pipe_active_pct"),
                 "profile": "profiles/k_gemm_plain_tma_2048_ncu.txt"}
        if rank == 0 and world == 1 and not args.skip_check:
            # its own error on 256 sampled entries, from the same C0 as the checked Ozaki step
            pc = torch.from_numpy(C0).to(dev)
            lib.mgemm("N", "N", n, n, n, alpha, dA.data_ptr(), n, dB.data_ptr(), n, beta, pc.data_ptr(), n,
                      engine="plain")
            torch.cuda.synchronize()
            plain_rows, plain_cols = np.random.default_rng(98).integers(0, n, 256), np.random.default_rng(97).integers(0, n, 256)
            plain["_check"] = (plain_rows, plain_cols, pc[torch.from_numpy(plain_cols).to(dev),
                                                        torch.from_numpy(plain_rows).to(dev)].cpu().numpy())
            del pc

    res = dict(value=value, ms=ms, launches=launches, moduli=moduli, phase_ms=phase.tolist(), e2e=e2e,
               e2e_pageable=e2e_pageable, plain=plain, clocks=clk.summary(),
               flops=flops, peaks=pk, peaks_kind=pk_kind, alpha=alpha, beta=beta, A=A, B=B, C0=C0,
               C=dC.cpu().numpy() if (rank == 0 and not args.skip_check) else None)
    lib.lib.mwblas_set_stream(None)
    return res


def cpu_baseline_leg(n, res):
    """rank 0, N=1: the oracle checks the GPU result on sampled entries, and the
    reference's CPU GEMM (or its port) is timed on a bounded sample."""
    orc = ge._load("oracle", os.path.join(ROOT, "oracle", "oracle.py"))
    o = orc.Oracle()
    out = {}
    if res.get("C") is not None:
        rng = np.random.default_rng(99)
        rows = rng.integers(0, n, 256)
        cols = rng.integers(0, n, 256)
        # after the timed steps C holds alpha*A*B + beta*C_prev; re-run one
        # checked step from C0 instead: compare entries of one step's output
        want = o.qgemm("N", "N", n, n, n, res["alpha"], res["A"], n, res["B"], n, res["beta"], res["C0"], n,
                       rows=rows, cols=cols)
        got = res["C_check"][cols, rows]
        op = orc.dd_abs(res["alpha"]) * n * orc.dd_absmax(res["A"]) * orc.dd_absmax(res["B"]) \
            + orc.dd_abs(res["beta"]) * orc.dd_absmax(res["C0"])
        out["normwise_err_sampled"] = orc.normwise_error(got, want, op)
        out["err_samples"] = 256
        pl = res.get("plain") or {}
        if "_check" in pl:
            prow, pcol, pgot = pl.pop("_check")
            pwant = o.qgemm("N", "N", n, n, n, res["alpha"], res["A"], n, res["B"], n, res["beta"], res["C0"], n,
                            rows=prow, cols=pcol)
            pl["normwise_err_vs_binary128"] = orc.normwise_error(pgot, pwant, op)
            pl["err_samples"] = 256
    # CPU timing on a bounded sample of the same workload
    t = time_reference_cpu(sample=(4096, 4096, 256), reps=1, single_thread=True)
    out["cpu"] = t
    return out


def _omp_threads(nt):
    """Sets the OpenMP team size of this process (libgomp: the oracle and the
    reference build share it); False where no libgomp is loaded."""
    try:
        import ctypes
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(nt))
        return True
    except (OSError, AttributeError):
        return False


def _cpu_gemm_runner(sample):
    """The reference's GEMM on the host cores: its own build where present
    (x86), else the C port of its algorithm; returns (runner, kind)."""
    m, n, k = sample
    rng = np.random.default_rng(5)
    mwb = ge._load("mwblas", os.path.join(ge.PKG, "mwblas.py"))
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    C = mwb.dd_matrix(rng, m, n)
    al, be = np.array([1.1, 0.0]), np.array([0.9, 0.0])
    ref_so = os.path.join(ROOT, "oracle", "_ref", "libmwblas_ref.so")
    try:
        if os.path.exists(ref_so):
            ref = mwb.MWBlas(ref_so, extensions=False)
            return (lambda: ref.mgemm("N", "N", m, n, k, al, A, m, B, k, be, C, m)), "reference"
    except OSError:
        pass
    orc = ge._load("oracle", os.path.join(ROOT, "oracle", "oracle.py"))
    o = orc.Oracle()
    import platform
    simd = 1 if platform.machine() in ("x86_64", "AMD64") else 0
    return (lambda: o.port_mgemm("N", "N", m, n, k, al, A, m, B, k, be, C, m, simd_order=simd)), "port"


def _best_seconds(runner, reps):
    runner()   # warm
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        runner()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best


def time_reference_cpu(sample=(4096, 4096, 256), reps=1, single_thread=False):
    """Times the reference's GEMM on the host cores with all threads (and, on
    request, with one thread on a 512 x 512 x 256 sample)."""
    m, n, k = sample
    runner, kind = _cpu_gemm_runner(sample)
    best = _best_seconds(runner, reps)
    cores = int(os.environ.get("OMP_NUM_THREADS", "0") or 0) or os.cpu_count()
    import platform
    out = {"value": 2.0 * m * n * k / best / 1e9, "unit": UNIT, "cores": cores, "kind": kind,
           "sample": f"mgemm_ {m}x{n}x{k} NN alpha=1.1 beta=0.9 ({platform.machine()}, min of {reps} after 1 warm-up,"
                     f" {best:.2f} s per call)"}
    if single_thread and _omp_threads(1):
        try:
            s1 = (512, 512, 256)
            r1, _ = _cpu_gemm_runner(s1)
            b1 = _best_seconds(r1, 3)
            out["single_thread"] = {"value": 2.0 * s1[0] * s1[1] * s1[2] / b1 / 1e9, "unit": UNIT, "cores": 1,
                                    "sample": "mgemm_ 512x512x256, min of 3 after 1 warm-up"}
        finally:
            _omp_threads(cores)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_GEMM)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-check", action="store_true")
    ap.add_argument("--workload", default="gemm", choices=WORKLOADS,
                    help="gemm: the headline line; the others measure one routine of the level-1/2/3 mix")
    ap.add_argument("--size", type=int, default=0,
                    help="problem size of a --workload line (n for dot/axpy, m=n for gemv, m for trsm, "
                         "n for gemm_fixed/gemm_plain); 0 keeps the default")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.workload != "gemm":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "secondary workloads have no CPU reference arm"}))
            return
        if not os.path.exists(os.path.join(ge.PKG, "libmwblas_gb300.so")):
            ge.build()
        run_workload(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    cfg = {"workload": f"mgemm_ {args.n}x{args.n}x{args.n} NN, random double-double alpha/beta (|.| in [0.5,2]), "
                       "A,B,C hi~U[-1,1) lo=hi*2^-53*U[-1,1)",
           "m": args.n, "n": args.n, "k": args.n, "api": "mgemm_64_ (engine chosen by the library: AUTO)",
           "engine": "ozaki-II CRT, tcgen05 kind::f16 residue GEMMs",
           "l2": "operands 1 GiB each, larger than the 129 MB L2", "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        steps = []
        for _ in range(args.warmup):
            time_reference_cpu(reps=1)
        for i in range(args.steps):
            steps.append(time_reference_cpu(reps=1, single_thread=(i == args.steps - 1)))
        v = float(np.median([s["value"] for s in steps]))
        cb = dict(steps[-1])
        cb["value"] = v
        cb["sample"] += f"; median of {args.steps} steps"
        # the rate does not hinge on the K = 256 slab: on 8 x86 cores the reference's own
        # build ran 17.2 GFLOP/s at 2048x2048x256 and 16.4 at 1536^3
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 2.0 * 4096 * 4096 * 256 / v / 1e6,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64x2 (double-double)",
                "data": "synthetic",
                "config": dict(cfg, sample="4096x4096x256 sample of the 8192^3 workload",
                               engine="the reference's mgemm_ on the host cores (OpenMP)"),
                "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    ge.build() if rank == 0 and not os.path.exists(os.path.join(ge.PKG, "libmwblas_gb300.so")) else None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = run_ours(args, rank, world, local_rank)
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    # correctness check data: one step from the original C
    import torch
    mwb = ge._load("mwblas", os.path.join(ge.PKG, "mwblas.py"))
    lib = mwb.MWBlas(os.path.join(ge.PKG, "libmwblas_gb300.so"))
    cpu = None
    if world == 1 and not args.skip_check:
        dA = torch.from_numpy(res["A"]).cuda()
        dB = torch.from_numpy(res["B"]).cuda()
        dC = torch.from_numpy(res["C0"]).cuda()
        n = args.n
        lib.mgemm("N", "N", n, n, n, res["alpha"], dA.data_ptr(), n, dB.data_ptr(), n, res["beta"], dC.data_ptr(), n)
        torch.cuda.synchronize()
        res["C_check"] = dC.cpu().numpy()
        del dA, dB, dC
        cpu = cpu_baseline_leg(args.n, res)

    pk, pk_kind = res["peaks"], res["peaks_kind"]
    n = args.n
    # Roofline of the dominant kernel (the tcgen05 residue GEMM on CTA pairs, one launch
    # per step): algorithmic fp16 tensor flops per launch = moduli * 2*m*n*k
    # (the padded tile work is not counted), over its CUDA-event duration.
    tc_ms = res["phase_ms"][2]
    tc_flops = res["moduli"] * 2.0 * n * n * n
    peak_tf = pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
    achieved = tc_flops / (tc_ms * 1e-3) / 1e12 if tc_ms > 0 else None
    roof = {"bound": "tensor",
            "kernel": "k_oz_gemm_tc_2sm (tcgen05.mma.cta_group::2 kind::f16, 256x256 tiles on SM pairs, "
                      "fp32 accumulate in TMEM)",
            "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
            "frac": (achieved / peak_tf) if achieved else None,
            "peak_kind": f"{pk_kind} bf16 dense, sustained figure (MEASURED_PEAKS.json)",
            "traffic": tc_traffic_from_profile(), "algorithmic_flops_per_launch": tc_flops,
            "kernel_ms": tc_ms,
            "step_phase_ms": dict(zip(["exponent_scan", "residues", "residue_gemm", "reconstruct"],
                                      res["phase_ms"]))}
    line = {"metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64x2 (double-double); residue GEMMs fp16 x fp16 -> fp32 exact",
            "data": "synthetic (seeded, reference value distribution)", "config": cfg,
            "e2e": res["e2e"], "e2e_pageable": res["e2e_pageable"], "gpu_launches": int(res["launches"]),
            "clocks": res["clocks"],
            "roofline": roof, "ozaki": {"moduli": res["moduli"], "bits": 106},
            "plain_fp64_eft": res["plain"]}
    if cpu:
        line["cpu_baseline"] = cpu["cpu"]
        if "normwise_err_sampled" in cpu:
            line["accuracy"] = {"normwise_err_vs_binary128": cpu["normwise_err_sampled"],
                                "sampled_entries": cpu["err_samples"], "gate": 1e-30}
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def plain_profile():
    """fp64_inst_per_mac / fp64_pipe_active_pct lines of the FP64 kernel's ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_gemm_plain_tma_2048_ncu.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            for key in ("fp64_inst_per_mac", "fp64_pipe_active_pct"):
                if line.startswith(key + ":"):
                    out[key] = float(line.split(":")[1].strip())
    return out


def tc_traffic_from_profile():
    return traffic_from_profile("k_oz_gemm_tc_2sm_4096_ncu.txt", "dram_bytes_per_launch_8192")


def traffic_from_profile(name, key="dram_bytes_per_launch"):
    """DRAM bytes (read + write) per launch recorded by an ncu capture in
    profiles/ (a `key: value` line), or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            return float(line.split(":")[1].strip())
    return None


# ---------------------------------------------------------------------------
# Secondary workloads (--workload ...): the level-1/2/3 mix and the batched
# workloads, each printed as one JSON line of the same shape as the headline.
# ---------------------------------------------------------------------------

WORKLOADS = ("gemm", "stress", "gemm_fp64", "wgemm", "gemm_t", "gemm_fixed", "gemm_plain", "syrk", "herk", "trsm", "gemv",
             "gemv_t", "dot",
             "axpy", "scal", "copy", "swap", "iamax", "batched_gemm", "batched_trsm", "gemmtr", "symm", "syr2k",
             "trmm", "wtrsm", "sbmv", "spmv", "tbsv")


def _dev_dd(torch, shape, gen, dev, cplx_=False):
    """Device DD array (..., 2) [(..., 2, 2) complex]: hi ~ U[-1,1), lo = hi*2^-53*U[-1,1), renormalised."""
    def one():
        hi = torch.rand(shape, generator=gen, device=dev, dtype=torch.float64) * 2 - 1
        lo = hi * 2.0 ** -53 * (torch.rand(shape, generator=gen, device=dev, dtype=torch.float64) * 2 - 1)
        s = hi + lo
        return torch.stack([s, lo - (s - hi)], -1)
    return torch.stack([one(), one()], -2) if cplx_ else one()


def _timed(torch, fn, steps, warmup, stream, reset=None, gpu=0):
    """Per-step CUDA events on the library's stream; `reset` runs between steps, untimed."""
    for _ in range(warmup):
        if reset:
            reset()
        fn()
    torch.cuda.synchronize()
    ms = 0.0
    with ClockSampler(gpu) as clk:
        for _ in range(steps):
            if reset:
                reset()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
    return ms / steps, clk.summary()


def run_workload(args):
    import torch
    mwb = ge._load("mwblas", os.path.join(ge.PKG, "mwblas.py"))
    orc = ge._load("oracle", os.path.join(ROOT, "oracle", "oracle.py"))
    lib = mwb.MWBlas(os.path.join(ge.PKG, "libmwblas_gb300.so"))
    o = orc.Oracle() if not args.skip_check else None
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    lib.lib.mwblas_set_stream(stream.cuda_stream)
    gen = torch.Generator(device=dev)
    gen.manual_seed(4321)
    rng = np.random.default_rng(4321)
    pk, pk_kind = peaks()
    w = args.workload
    hb = lambda t: t.cpu().numpy()
    al = np.array([1.25, 1.25 * 2.0 ** -55])
    be = np.array([-0.75, 0.75 * 2.0 ** -56])
    check = {}
    roof = None
    l0 = lib.lib.mwblas_launch_count()

    if w == "stress":
        # Exponent-spread stress input: A(i,:) = U[1,2)*sign * 2^e_i, B(:,j) = ... * 2^f_j,
        # e_i, f_j uniform integers in [-30, 30]; Ozaki engine at n^3.
        n = args.n
        def spread(row_scaled):
            u = torch.rand((n, n), generator=gen, device=dev, dtype=torch.float64) * 2 - 1
            mant = torch.where(u < 0, -1.0, 1.0) * (1 + u.abs())
            lo = mant * 2.0 ** -53 * (torch.rand((n, n), generator=gen, device=dev, dtype=torch.float64) * 2 - 1)
            hi = mant + lo
            lo = lo - (hi - mant)
            sc = torch.pow(2.0, torch.randint(-30, 31, (n,), generator=gen, device=dev).to(torch.float64))
            sc = sc[None, :] if row_scaled else sc[:, None]     # storage [column, row]
            return torch.stack([hi * sc, lo * sc], -1).contiguous()
        A, B = spread(True), spread(False)
        C = _dev_dd(torch, (n, n), gen, dev)
        C0 = C.clone()
        fn = lambda: lib.mgemm("N", "N", n, n, n, al, A.data_ptr(), n, B.data_ptr(), n, be, C.data_ptr(), n,
                               engine="ozaki")
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit, metric = 2.0 * n ** 3 / ms / 1e6, "DD-GFLOP/s", f"DD-GEMM GFLOP/s n={n} exponent-spread stress, Ozaki"
        cfg = {"workload": f"mgemm_ {n}^3 NN, A rows / B columns scaled by 2^e, e ~ U{{-30..30}}", "engine": "ozaki"}
        check["moduli"] = int(lib.lib.mwblas_last_ozaki_moduli())
        if o:
            C.copy_(C0)
            fn()
            rows, cols = rng.integers(0, n, 256), rng.integers(0, n, 256)
            hA, hB, hC0 = hb(A), hb(B), hb(C0)
            want = o.qgemm("N", "N", n, n, n, al, hA, n, hB, n, be, hC0, n, rows=rows, cols=cols)
            got = hb(C)[cols, rows]
            op = orc.dd_abs(al) * n * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC0)
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
            # componentwise view: error relative to |alpha| sum_p |a_ip||b_pj| of the sampled entries
            check["samples"] = 256
    elif w == "gemm_fp64":
        # FP64 operands (lo = 0, hi ~ U[-1,1): the reference fuzz's real64x2(2u-1)) through the
        # drop-in mgemm_64_ at n^3: the moduli count follows from their significant width
        n = args.n
        A = _dev_dd(torch, (n, n), gen, dev)
        B = _dev_dd(torch, (n, n), gen, dev)
        A[..., 1] = 0.0
        B[..., 1] = 0.0
        C = _dev_dd(torch, (n, n), gen, dev)
        C0 = C.clone()
        lib.lib.mwblas_set_gemm_engine(0)
        fn = lambda: lib.mgemm("N", "N", n, n, n, al, A.data_ptr(), n, B.data_ptr(), n, be, C.data_ptr(), n)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = 2.0 * n ** 3 / ms / 1e6, "DD-GFLOP/s"
        metric = f"DD-GEMM GFLOP/s n={n} NN, FP64 operands (lo = 0), moduli from the operands' width"
        cfg = {"workload": f"mgemm_64_ {n}^3 NN, A and B with lo = 0, hi ~ U[-1,1)", "engine": "AUTO"}
        check["moduli"] = int(lib.lib.mwblas_last_ozaki_moduli())
        check["bits"] = [int(lib.lib.mwblas_last_ozaki_bits(0)), int(lib.lib.mwblas_last_ozaki_bits(1))]
        if o:
            C.copy_(C0)
            fn()
            rows, cols = rng.integers(0, n, 256), rng.integers(0, n, 256)
            hA, hB, hC0 = hb(A), hb(B), hb(C0)
            want = o.qgemm("N", "N", n, n, n, al, hA, n, hB, n, be, hC0, n, rows=rows, cols=cols)
            op = orc.dd_abs(al) * n * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC0)
            check["normwise_err_sampled"] = orc.normwise_error(hb(C)[cols, rows], want, op)
            check["samples"] = 256
    elif w in ("gemm_fixed", "gemm_plain"):
        # one engine forced, n^3 NN (default n = 4096)
        eng = w.split("_")[1]
        n = args.size or 4096
        A = _dev_dd(torch, (n, n), gen, dev)
        B = _dev_dd(torch, (n, n), gen, dev)
        C = _dev_dd(torch, (n, n), gen, dev)
        C0 = C.clone()
        fn = lambda: lib.mgemm("N", "N", n, n, n, al, A.data_ptr(), n, B.data_ptr(), n, be, C.data_ptr(), n,
                               engine=eng)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = 2.0 * n ** 3 / ms / 1e6, "DD-GFLOP/s"
        metric = f"DD-GEMM GFLOP/s n={n} NN, {eng} engine"
        cfg = {"workload": f"mgemm_{eng}_64_ {n}^3 NN"}
        if o:
            C.copy_(C0)
            fn()
            rows, cols = rng.integers(0, n, 128), rng.integers(0, n, 128)
            hA, hB, hC0 = hb(A), hb(B), hb(C0)
            want = o.qgemm("N", "N", n, n, n, al, hA, n, hB, n, be, hC0, n, rows=rows, cols=cols)
            op = orc.dd_abs(al) * n * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC0)
            check["normwise_err_sampled"] = orc.normwise_error(hb(C)[cols, rows], want, op)
    elif w in ("wgemm", "gemm_t"):
        # complex GEMM at 4096^3 NN, or the real GEMM at n^3 with both operands transposed
        cx = w == "wgemm"
        n = 4096 if cx else args.n
        A = _dev_dd(torch, (n, n), gen, dev, cplx_=cx)
        B = _dev_dd(torch, (n, n), gen, dev, cplx_=cx)
        C = _dev_dd(torch, (n, n), gen, dev, cplx_=cx)
        C0 = C.clone()
        ca = np.array([al, be])            # complex alpha = al + i*be
        cb = np.array([be, al])
        if cx:
            fn = lambda: lib.wgemm("N", "N", n, n, n, ca, A.data_ptr(), n, B.data_ptr(), n, cb, C.data_ptr(), n)
            value_flops = 8.0 * n ** 3
            metric = "complex DD-GEMM GFLOP/s n=4096 NN (8n^3 real flops)"
            cfg = {"workload": "wgemm_ 4096^3 NN, complex double-double alpha/beta"}
        else:
            fn = lambda: lib.mgemm("T", "T", n, n, n, al, A.data_ptr(), n, B.data_ptr(), n, be, C.data_ptr(), n)
            value_flops = 2.0 * n ** 3
            metric = f"DD-GEMM GFLOP/s n={n} TT"
            cfg = {"workload": f"mgemm_ {n}^3 TT"}
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = value_flops / ms / 1e6, "DD-GFLOP/s"
        if o:
            C.copy_(C0)
            fn()
            rows, cols = rng.integers(0, n, 128), rng.integers(0, n, 128)
            hA, hB, hC0 = hb(A), hb(B), hb(C0)
            if cx:
                want = o.qwgemm("N", "N", n, n, n, ca, hA, n, hB, n, cb, hC0, n, rows=rows, cols=cols)
                op = (orc.dd_abs(al) + orc.dd_abs(be)) * 2 * n * orc.dd_absmax(hA) * orc.dd_absmax(hB) \
                    + 2 * (orc.dd_abs(al) + orc.dd_abs(be)) * orc.dd_absmax(hC0)
            else:
                want = o.qgemm("T", "T", n, n, n, al, hA, n, hB, n, be, hC0, n, rows=rows, cols=cols)
                op = orc.dd_abs(al) * n * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC0)
            got = hb(C)[cols, rows]
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w == "syrk":
        n, k = 8192, 2048
        A = _dev_dd(torch, (k, n), gen, dev)          # n x k, lda = n
        C = _dev_dd(torch, (n, n), gen, dev)
        C0 = C.clone()
        fn = lambda: lib.msyrk("U", "N", n, k, al, A.data_ptr(), n, be, C.data_ptr(), n)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = n * (n + 1) * k / ms / 1e6, "DD-GFLOP/s"
        metric = "DD-SYRK GFLOP/s n=8192 k=2048 upper (n(n+1)k flops)"
        cfg = {"workload": "msyrk_ U N n=8192 k=2048"}
        if o:
            C.copy_(C0)
            fn()
            i = rng.integers(0, n, 256)
            j = rng.integers(0, n, 256)
            rows, cols = np.minimum(i, j), np.maximum(i, j)
            hA, hC0 = hb(A), hb(C0)
            want = o.qgemm("N", "T", n, n, k, al, hA, n, hA, n, be, hC0, n, rows=rows, cols=cols)
            got = hb(C)[cols, rows]
            op = orc.dd_abs(al) * k * orc.dd_absmax(hA) ** 2 + orc.dd_abs(be) * orc.dd_absmax(hC0)
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w == "herk":
        n, k = 4096, 1024
        A = _dev_dd(torch, (k, n), gen, dev, cplx_=True)
        C = _dev_dd(torch, (n, n), gen, dev, cplx_=True)
        C0 = C.clone()
        fn = lambda: lib.wherk("U", "N", n, k, al, A.data_ptr(), n, be, C.data_ptr(), n)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = 4.0 * n * (n + 1) * k / ms / 1e6, "DD-GFLOP/s"
        metric = "DD-HERK GFLOP/s n=4096 k=1024 upper (4n(n+1)k real flops)"
        cfg = {"workload": "wherk_ U N n=4096 k=1024 complex"}
        if o:
            C.copy_(C0)
            fn()
            i = rng.integers(0, n, 256)
            j = rng.integers(0, n, 256)
            rows, cols = np.minimum(i, j), np.maximum(i, j)
            off = rows != cols
            rows, cols = rows[off], cols[off]
            hA, hC0 = hb(A), hb(C0)
            ca = np.array([al, [0.0, 0.0]])
            cb = np.array([be, [0.0, 0.0]])
            want = o.qwgemm("N", "C", n, n, k, ca, hA, n, hA, n, cb, hC0, n, rows=rows, cols=cols)
            got = hb(C)[cols, rows]
            op = 2 * (orc.dd_abs(al) * k * orc.dd_absmax(hA) ** 2 + orc.dd_abs(be) * orc.dd_absmax(hC0))
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w == "trsm":
        m, nr = (args.size or 4096), 1024
        A = _dev_dd(torch, (m, m), gen, dev)
        A[..., 0] /= m
        A[..., 1] /= m
        d = torch.arange(m, device=dev)
        dg = m * (1 + torch.rand(m, generator=gen, device=dev, dtype=torch.float64))
        A[d, d, 0] = dg
        A[d, d, 1] = 0.0
        B = _dev_dd(torch, (nr, m), gen, dev)
        B0 = B.clone()
        fn = lambda: lib.mtrsm("L", "L", "N", "N", m, nr, al, A.data_ptr(), m, B.data_ptr(), m)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: B.copy_(B0))
        value, unit = float(m) * m * nr / ms / 1e6, "DD-GFLOP/s"
        metric = f"DD-TRSM GFLOP/s LLNN m={m} nrhs=1024 (m^2 nrhs flops)"
        cfg = {"workload": f"mtrsm_ L L N N m={m} n=1024, diag U[m,2m], off-diagonal U[-1,1)/m"}
        if o:
            B.copy_(B0)
            fn()
            cols = rng.choice(nr, 4, replace=False)
            hA = hb(A)
            want = np.ascontiguousarray(hb(B0)[cols])
            o.qtrsm("L", "L", "N", "N", m, len(cols), al, hA, m, want, m)
            got = hb(B)[cols]
            check["normwise_err_sampled"] = orc.normwise_error(got, want, orc.dd_abs(al) * orc.dd_absmax(hb(B0)))
            check["columns_checked"] = len(cols)
    elif w == "gemmtr":
        n, k = 8192, 2048
        A = _dev_dd(torch, (k, n), gen, dev)           # n x k
        B = _dev_dd(torch, (n, k), gen, dev)           # k x n
        C = _dev_dd(torch, (n, n), gen, dev)
        C0 = C.clone()
        fn = lambda: lib.gemmtr("U", "N", "N", n, k, al, A.data_ptr(), n, B.data_ptr(), k, be, C.data_ptr(), n)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = n * (n + 1) * k / ms / 1e6, "DD-GFLOP/s"
        metric = "DD-GEMMTR GFLOP/s n=8192 k=2048 upper (n(n+1)k flops)"
        cfg = {"workload": "mgemmtr_ U N N n=8192 k=2048"}
        if o:
            C.copy_(C0)
            fn()
            i, j = rng.integers(0, n, 256), rng.integers(0, n, 256)
            rows, cols = np.minimum(i, j), np.maximum(i, j)
            hA, hB, hC0 = hb(A), hb(B), hb(C0)
            want = o.qgemm("N", "N", n, n, k, al, hA, n, hB, k, be, hC0, n, rows=rows, cols=cols)
            got = hb(C)[cols, rows]
            op = orc.dd_abs(al) * k * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC0)
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w == "symm":
        m = n = 8192
        A = _dev_dd(torch, (m, m), gen, dev)           # symmetric, upper triangle used
        B = _dev_dd(torch, (n, m), gen, dev)
        C = _dev_dd(torch, (n, m), gen, dev)
        C0 = C.clone()
        fn = lambda: lib.symm("msymm", "L", "U", m, n, al, A.data_ptr(), m, B.data_ptr(), m, be, C.data_ptr(), m)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = 2.0 * m * m * n / ms / 1e6, "DD-GFLOP/s"
        metric = "DD-SYMM GFLOP/s m=n=8192 side L upper (2m^2n flops)"
        cfg = {"workload": "msymm_ L U m=n=8192"}
        if o:
            C.copy_(C0)
            fn()
            hA = hb(A)
            iu = np.triu_indices(m)   # array [col, row]: row <= col is the stored upper triangle
            full = np.empty_like(hA)
            full[iu[1], iu[0]] = hA[iu[1], iu[0]]
            full[iu[0], iu[1]] = hA[iu[1], iu[0]]
            rows, cols = rng.integers(0, m, 256), rng.integers(0, n, 256)
            hB, hC0 = hb(B), hb(C0)
            want = o.qgemm("N", "N", m, n, m, al, full, m, hB, m, be, hC0, m, rows=rows, cols=cols)
            got = hb(C)[cols, rows]
            op = orc.dd_abs(al) * m * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC0)
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w == "syr2k":
        n, k = 8192, 2048
        A = _dev_dd(torch, (k, n), gen, dev)
        B = _dev_dd(torch, (k, n), gen, dev)
        C = _dev_dd(torch, (n, n), gen, dev)
        C0 = C.clone()
        fn = lambda: lib.syr2k("msyr2k", "U", "N", n, k, al, A.data_ptr(), n, B.data_ptr(), n, be, C.data_ptr(), n)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: C.copy_(C0))
        value, unit = 2.0 * n * (n + 1) * k / ms / 1e6, "DD-GFLOP/s"
        metric = "DD-SYR2K GFLOP/s n=8192 k=2048 upper (2n(n+1)k flops)"
        cfg = {"workload": "msyr2k_ U N n=8192 k=2048"}
        if o:
            C.copy_(C0)
            fn()
            i, j = rng.integers(0, n, 256), rng.integers(0, n, 256)
            rows, cols = np.minimum(i, j), np.maximum(i, j)
            hA, hB, hC0 = hb(A), hb(B), hb(C0)
            # both products in one binary128 sum: [A B] [B A]^T
            AB = np.ascontiguousarray(np.concatenate([hA, hB], axis=0))
            BA = np.ascontiguousarray(np.concatenate([hB, hA], axis=0))
            want = o.qgemm("N", "T", n, n, 2 * k, al, AB, n, BA, n, be, hC0, n, rows=rows, cols=cols)
            got = hb(C)[cols, rows]
            op = 2 * orc.dd_abs(al) * k * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC0)
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w == "trmm":
        m, n = 8192, 4096
        A = _dev_dd(torch, (m, m), gen, dev)           # upper triangle used, non-unit
        B = _dev_dd(torch, (n, m), gen, dev)
        B0 = B.clone()
        fn = lambda: lib.trxm("mtrmm", "L", "U", "N", "N", m, n, al, A.data_ptr(), m, B.data_ptr(), m)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: B.copy_(B0))
        value, unit = float(m) * m * n / ms / 1e6, "DD-GFLOP/s"
        metric = "DD-TRMM GFLOP/s m=8192 n=4096 LUNN (m^2 n flops)"
        cfg = {"workload": "mtrmm_ L U N N m=8192 n=4096"}
        if o:
            B.copy_(B0)
            fn()
            hA = hb(A)
            tri = np.zeros_like(hA)
            iu = np.triu_indices(m)
            tri[iu[1], iu[0]] = hA[iu[1], iu[0]]
            rows, cols = rng.integers(0, m, 256), rng.integers(0, n, 256)
            hB0 = hb(B0)
            want = o.qgemm("N", "N", m, n, m, al, tri, m, hB0, m, np.zeros(2), np.zeros_like(hB0), m,
                           rows=rows, cols=cols)
            got = hb(B)[cols, rows]
            op = orc.dd_abs(al) * m * orc.dd_absmax(hA) * orc.dd_absmax(hB0)
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w == "wtrsm":
        m, nr = (args.size or 4096), 1024
        A = _dev_dd(torch, (m, m), gen, dev, cplx_=True) / m
        d = torch.arange(m, device=dev)
        A[d, d, 0, 0] = 1 + torch.rand(m, generator=gen, device=dev, dtype=torch.float64)
        A[d, d, 0, 1] = 0.0
        B = _dev_dd(torch, (nr, m), gen, dev, cplx_=True)
        B0 = B.clone()
        ca = np.array([al, [0.5, 0.0]])
        fn = lambda: lib.trxm("wtrsm", "L", "L", "N", "N", m, nr, ca, A.data_ptr(), m, B.data_ptr(), m)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: B.copy_(B0))
        value, unit = 4.0 * m * m * nr / ms / 1e6, "DD-GFLOP/s"
        metric = f"complex DD-TRSM GFLOP/s LLNN m={m} nrhs=1024 (4 m^2 nrhs real flops)"
        cfg = {"workload": f"wtrsm_ L L N N m={m} n=1024, diag U[1,2), off-diagonal U[-1,1)/m"}
        if o:
            B.copy_(B0)
            fn()
            # residual op(A) X - alpha B at 256 sampled entries, in binary128
            hA, X, hB0 = hb(A), hb(B), hb(B0)
            tri = np.zeros_like(hA)
            il = np.tril_indices(m)
            tri[il[1], il[0]] = hA[il[1], il[0]]
            rows, cols = rng.integers(0, m, 256), rng.integers(0, nr, 256)
            one, zero = np.array([[1.0, 0.0], [0.0, 0.0]]), np.zeros((2, 2))
            AX = o.qwgemm("N", "N", m, nr, m, one, tri, m, X, m, zero, np.zeros_like(X), m, rows=rows, cols=cols)
            # alpha * B0 at the same entries: a k = 1 product with a 1 x 1 one
            eye1 = np.ascontiguousarray(one.reshape(1, 1, 2, 2))
            rhs = np.stack([o.qwgemm("N", "N", m, 1, 1, ca, np.ascontiguousarray(hB0[c:c + 1]), m, eye1, 1, zero,
                                     np.zeros((1, m, 2, 2)), m, rows=np.array([r]), cols=np.array([0]))[0]
                            for r, c in zip(rows, cols)])
            scale = m * orc.dd_absmax(tri) * orc.dd_absmax(X) + orc.dd_abs(ca) * orc.dd_absmax(hB0)
            check["normwise_residual_sampled"] = orc.normwise_error(AX, rhs, scale)
            check["entries_checked"] = 256
    elif w in ("gemv", "gemv_t"):
        # square GEMV, op(A) = A (a thread per row) or A^T (a block per column)
        tr = "T" if w == "gemv_t" else "N"
        m = n = args.size or 16384
        A = _dev_dd(torch, (n, m), gen, dev)
        x = _dev_dd(torch, (n,), gen, dev)
        y = _dev_dd(torch, (m,), gen, dev)
        y0 = y.clone()
        fn = lambda: lib.mgemv(tr, m, n, al, A.data_ptr(), m, x.data_ptr(), 1, be, y.data_ptr(), 1)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: y.copy_(y0))
        nbytes = 16.0 * (m * n + n + 2 * m)
        value, unit = nbytes / ms / 1e6, "GB/s"
        metric = f"DD-GEMV{'-T' if tr == 'T' else ''} HBM GB/s m=n={n} (16(mn+n+2m) bytes)"
        cfg = {"workload": f"mgemv_ {tr} m=n={n} incx=incy=1"}
        roof = {"bound": "hbm", "achieved": value, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": value / pk["hbm_gbs"], "peak_kind": pk_kind, "traffic": None}
        if o:
            y.copy_(y0)
            fn()
            rows = np.sort(rng.choice(m, 64, replace=False))
            want = hb(y0)[rows].copy()
            if tr == "N":
                sub = np.ascontiguousarray(hb(A[:, torch.as_tensor(rows, device=dev)]))
                o.qgemv("N", len(rows), n, al, sub, len(rows), hb(x), 1, be, want, 1)
            else:   # entries rows of y = columns of A
                sub = np.ascontiguousarray(hb(A[torch.as_tensor(rows, device=dev)]))
                o.qgemv("T", m, len(rows), al, sub, m, hb(x), 1, be, want, 1)
            got = hb(y)[rows]
            amax = float(A[..., 0].abs().max())
            op = orc.dd_abs(al) * n * amax * orc.dd_absmax(hb(x)) + orc.dd_abs(be) * orc.dd_absmax(hb(y0))
            check["normwise_err_sampled"] = orc.normwise_error(got, want, op)
    elif w in ("sbmv", "spmv"):
        # symmetric band (k = 16, n = 2^22) / packed (n = 16384) matrix-vector
        # products, A read in place from its band or packed storage
        band = w == "sbmv"
        n = args.size or ((1 << 22) if band else 16384)
        k = 16
        nst = n * (k + 1) if band else n * (n + 1) // 2
        A = _dev_dd(torch, (n, k + 1) if band else (nst,), gen, dev)
        x = _dev_dd(torch, (n,), gen, dev)
        y = _dev_dd(torch, (n,), gen, dev)
        y0 = y.clone()
        if band:
            fn = lambda: lib.l2("msbmv", "U", n, k, al, (A.data_ptr(),), k + 1, (x.data_ptr(),), 1, be,
                                (y.data_ptr(),), 1)
        else:
            fn = lambda: lib.l2("mspmv", "U", n, al, (A.data_ptr(),), (x.data_ptr(),), 1, be, (y.data_ptr(),), 1)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: y.copy_(y0))
        nbytes = 16.0 * (nst + 3 * n)
        value, unit = nbytes / ms / 1e6, "GB/s"
        metric = (f"DD-{'SBMV' if band else 'SPMV'} HBM GB/s n={n}" + (f" k={k}" if band else "")
                  + " (16(stored + 3n) bytes)")
        cfg = {"workload": f"m{w}_ U n={n}" + (f" k={k}" if band else "") + " incx=incy=1"}
        # traffic: the band kernel's, or the two packed halves' per call, at these sizes
        traffic = None
        if not args.size:
            traffic = traffic_from_profile("k_sbmv_tile_n4M_k16_ncu.txt" if band else "mspmv_16384_launches.txt")
        roof = {"bound": "hbm", "achieved": value, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": value / pk["hbm_gbs"], "peak_kind": pk_kind, "traffic": traffic}
        if o:
            y.copy_(y0)
            fn()
            rows = np.sort(rng.choice(n, 32, replace=False))
            hx, hy0, hy = hb(x), hb(y0), hb(y)
            got, want = [], []
            for r in rows:
                c0, c1 = (max(0, r - k), min(n - 1, r + k)) if band else (0, n - 1)
                cs = np.arange(c0, c1 + 1)
                i, j = np.minimum(cs, r), np.maximum(cs, r)           # stored upper entry (i <= j)
                if band:
                    idx = torch.as_tensor(j * (k + 1) + (k + i - j), device=dev)
                    row = A.reshape(-1, 2)[idx]
                else:
                    row = A[torch.as_tensor(i + j * (j + 1) // 2, device=dev)]
                rv = np.ascontiguousarray(hb(row)[:, None, :])           # 1 x len, lda 1
                yr = hy0[r:r + 1].copy()
                o.qgemv("N", 1, len(cs), al, rv, 1, np.ascontiguousarray(hx[c0:c1 + 1]), 1, be, yr, 1)
                want.append(yr[0])
                got.append(hy[r])
            op = orc.dd_abs(al) * (2 * k + 1 if band else n) * orc.dd_absmax(hb(A[:1 << 20])) * orc.dd_absmax(hx) \
                + orc.dd_abs(be) * orc.dd_absmax(hy0)
            check["normwise_err_sampled"] = orc.normwise_error(np.array(got), np.array(want), op)
            check["rows_checked"] = len(rows)
    elif w == "tbsv":
        # lower band triangular solve, n = 2^20, k = 16, A read in place from its band
        n = args.size or (1 << 20)
        k = 16
        A = _dev_dd(torch, (n, k + 1), gen, dev)                  # band storage: row 0 is the diagonal
        A[:, 1:] /= 4 * k
        A[:, 0, 0] = 1.0 + torch.rand(n, generator=gen, device=dev, dtype=torch.float64)
        A[:, 0, 1] = 0.0
        x = _dev_dd(torch, (n,), gen, dev)
        x0 = x.clone()
        fn = lambda: lib.l2("mtbsv", "L", "N", "N", n, k, (A.data_ptr(),), k + 1, (x.data_ptr(),), 1)
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: x.copy_(x0))
        nbytes = 16.0 * (n * (k + 1) + 2 * n)
        value, unit = nbytes / ms / 1e6, "GB/s"
        metric = f"DD-TBSV GB/s n={n} k={k} lower (16(n(k+1) + 2n) bytes; one warp, sequential in n)"
        cfg = {"workload": f"mtbsv_ L N N n={n} k={k} incx=1, diagonal U[1,2), off-diagonal U[-1,1)/(4k)"}
        if o:
            x.copy_(x0)
            fn()
            hA, hx, hbv = hb(A), hb(x), hb(x0)
            rows = np.sort(rng.choice(n, 32, replace=False))
            got, want = [], []
            for r in rows:
                c0 = max(0, r - k)
                cs = np.arange(c0, r + 1)
                row = hA[cs, r - cs]                                   # A(r, c) = AB(r - c, c)
                rv = np.ascontiguousarray(row[:, None, :])
                res = np.zeros((1, 2))
                o.qgemv("N", 1, len(cs), np.array([1.0, 0.0]), rv, 1, np.ascontiguousarray(hx[c0:r + 1]), 1,
                        np.array([0.0, 0.0]), res, 1)
                got.append(res[0])
                want.append(hbv[r])
            scale = (k + 1) * orc.dd_absmax(hA[:4096]) * orc.dd_absmax(hx)
            check["normwise_residual_sampled"] = orc.normwise_error(np.array(got), np.array(want), scale)
            check["rows_checked"] = len(rows)
    elif w in ("scal", "copy", "swap", "iamax"):
        # HBM-bound level-1 moves at n = 2^28 (SCAL bit-exact, FP64-bound by its operation sequence)
        n = args.size or (1 << 28)
        x = _dev_dd(torch, (n,), gen, dev)
        y = _dev_dd(torch, (n,), gen, dev) if w in ("copy", "swap") else None
        x0 = x.clone() if w == "scal" else None
        if w == "scal":
            fn = lambda: lib.mscal(n, al, x.data_ptr(), 1)
            reset, nbytes = (lambda: x.copy_(x0)), 32.0 * n
        elif w == "copy":
            fn = lambda: lib.mcopy(n, x.data_ptr(), 1, y.data_ptr(), 1)
            reset, nbytes = None, 32.0 * n
        elif w == "swap":
            fn = lambda: lib.mswap(n, x.data_ptr(), 1, y.data_ptr(), 1)
            reset, nbytes = None, 64.0 * n
        else:
            out = {}
            fn = lambda: out.__setitem__("i", lib.imamax(n, x.data_ptr(), 1))
            reset, nbytes = None, 16.0 * n
        ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=reset)
        value, unit = nbytes / ms / 1e6, "GB/s"
        metric = f"DD-{w.upper()} HBM GB/s n={n} ({int(nbytes // n)}n bytes)"
        cfg = {"workload": f"{'i' if w == 'iamax' else 'm'}{w if w != 'iamax' else 'mamax'}_ n={n} inc=1"}
        roof = {"bound": "hbm" if w != "scal" else "fp64 (bit-exact operation sequence)", "achieved": value,
                "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": value / pk["hbm_gbs"], "peak_kind": pk_kind,
                "traffic": None}
        if w == "iamax" and o is not None:
            hx = hb(x)
            mag = np.abs(hx[:, 0])
            want = int(np.argmax(mag)) + 1
            check["index_matches_host_argmax_of_hi"] = (out["i"] == want)
    elif w in ("dot", "axpy"):
        n = args.size or (1 << 28)
        x = _dev_dd(torch, (n,), gen, dev)
        y = _dev_dd(torch, (n,), gen, dev)
        if w == "dot":
            out = {}
            fn = lambda: out.__setitem__("r", lib.mdot(n, x.data_ptr(), 1, y.data_ptr(), 1))
            ms, clk = _timed(torch, fn, args.steps, args.warmup, stream)
            nbytes = 32.0 * n
            metric = f"DD-DOT HBM GB/s n={n} (32n bytes)"
            cfg = {"workload": f"mdot_ n={n} incx=incy=1"}
            if o:
                hx, hy = hb(x), hb(y)
                want = o.qdot(n, hx, 1, hy, 1)
                got = np.array(out["r"]).reshape(1, 2)
                check["normwise_err"] = orc.normwise_error(got, np.asarray(want).reshape(1, 2),
                                                            n * orc.dd_absmax(hx) * orc.dd_absmax(hy))
        else:
            y0 = y.clone()
            fn = lambda: lib.maxpy(n, al, x.data_ptr(), 1, y.data_ptr(), 1)
            ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: y.copy_(y0))
            nbytes = 48.0 * n
            metric = f"DD-AXPY HBM GB/s n={n} (48n bytes)"
            cfg = {"workload": f"maxpy_ n={n} incx=incy=1"}
            if o:
                y.copy_(y0)
                fn()
                idx = torch.as_tensor(np.sort(rng.choice(n, 4096, replace=False)), device=dev)
                want = np.ascontiguousarray(hb(y0[idx]))
                o.qaxpy(len(idx), al, np.ascontiguousarray(hb(x[idx])), want)
                got = hb(y[idx])
                check["normwise_err_sampled"] = orc.normwise_error(got, want, orc.dd_abs(al) * orc.dd_absmax(hb(x[idx]))
                                                                   + orc.dd_absmax(hb(y0[idx])))
        value, unit = nbytes / ms / 1e6, "GB/s"
        roof = {"bound": "hbm", "achieved": value, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": value / pk["hbm_gbs"], "peak_kind": pk_kind, "traffic": None}
    elif w in ("batched_gemm", "batched_trsm"):
        cnt = 20000 if w == "batched_gemm" else 5000
        if w == "batched_gemm":
            dims = np.exp(rng.uniform(np.log(8), np.log(512), (cnt, 3))).round().astype(np.int64)
            m_, n_, k_ = dims[:, 0], dims[:, 1], dims[:, 2]
            sizes = np.stack([m_ * k_, k_ * n_, m_ * n_], 1)
        else:
            m_ = np.exp(rng.uniform(np.log(16), np.log(256), cnt)).round().astype(np.int64)
            n_ = rng.integers(1, 65, cnt)
            sizes = np.stack([m_ * m_, m_ * n_], 1)
        offs = np.concatenate([[0], np.cumsum(sizes.reshape(-1))])
        arena = _dev_dd(torch, (int(offs[-1]),), gen, dev)
        base = arena.data_ptr()
        ptr = lambda q: [base + 16 * int(v) for v in offs[q:-1:sizes.shape[1]]]
        if w == "batched_gemm":
            a_p, b_p, c_p = ptr(0), ptr(1), ptr(2)
            C0 = arena.clone()
            ta, tb = ["N"] * cnt, ["N"] * cnt
            alist, blist = [al] * cnt, [be] * cnt
            args_g = dict(ta=ta, tb=tb, m=m_, n=n_, k=k_, alpha=alist, a=a_p, lda=m_, b=b_p, ldb=k_, beta=blist,
                          c=c_p, ldc=m_)
            rc, chosen = lib.mgemm_grouped_tune(**args_g)
            assert rc == 0, lib.last_error()
            garr = lib._grouped_arrays(*[args_g[k] for k in ("ta", "tb", "m", "n", "k", "alpha", "a", "lda", "b",
                                                            "ldb", "beta", "c", "ldc")])
            gptrs = [x.ctypes.data for x in garr[1:]]
            fn = lambda: lib.lib.mgemm_grouped(garr[0], *gptrs)
            ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: arena.copy_(C0))
            value, unit = float(np.sum(2.0 * m_ * n_ * k_)) / ms / 1e6, "DD-GFLOP/s"
            metric = "batched DD-GEMM GFLOP/s, 20000 instances M,N,K log-uniform [8,512]"
            cfg = {"workload": "mgemm_grouped 20000 x NN, M,N,K ~ logU[8,512]", "split_k_min_chosen": chosen,
                   "tile_chosen": int(lib.lib.mwblas_grouped_tuned_tile()),
                   "tensor_core_min_size_chosen": int(lib.lib.mwblas_grouped_tuned_tensor_min()),
                   "tensor_core_pack_depth_chosen": int(lib.lib.mwblas_grouped_tuned_tensor_pack()),
                   "launch": "one CUDA graph per batch layout: the persistent integer-pipe kernel for the small "
                             "instances, the grouped tensor-core residue GEMMs (one per padding class) for those "
                             "with m, n >= the chosen size and k >= 64"}
            if o:
                arena.copy_(C0)
                fn()
                torch.cuda.synchronize()
                errs = []
                for t in rng.choice(cnt, 16, replace=False):
                    mm, nn, kk = int(m_[t]), int(n_[t]), int(k_[t])
                    seg = lambda q, r, c: hb(C0[int(offs[3 * t + q]):int(offs[3 * t + q]) + r * c]).reshape(c, r, 2)
                    hA, hB, hC = seg(0, mm, kk), seg(1, kk, nn), seg(2, mm, nn)
                    want = o.qgemm("N", "N", mm, nn, kk, al, hA, mm, hB, kk, be, hC.copy(), mm)
                    got = hb(arena[int(offs[3 * t + 2]):int(offs[3 * t + 2]) + mm * nn]).reshape(nn, mm, 2)
                    op = orc.dd_abs(al) * kk * orc.dd_absmax(hA) * orc.dd_absmax(hB) + orc.dd_abs(be) * orc.dd_absmax(hC)
                    errs.append(orc.normwise_error(got, want, op) / (max(10, 4 * kk) * orc.EPS_DD))
                check["max_err_over_tolerance_16_instances"] = float(max(errs))
        else:
            a_p, b_p = ptr(0), ptr(1)
            # lower-triangular, diagonally dominant: off-diagonal / n, diagonal U[n, 2n]
            for t in range(cnt):
                nn = int(m_[t])
                blk = arena[int(offs[2 * t]):int(offs[2 * t]) + nn * nn].view(nn, nn, 2)
                blk /= nn
            diag_idx = np.concatenate([offs[2 * t] + np.arange(int(m_[t])) * (int(m_[t]) + 1) for t in range(cnt)])
            dv = torch.as_tensor(diag_idx, device=dev)
            mt = torch.as_tensor(np.repeat(m_, m_).astype(np.float64), device=dev)
            arena[dv, 0] = mt * (1 + torch.rand(len(diag_idx), generator=gen, device=dev, dtype=torch.float64))
            arena[dv, 1] = 0.0
            B0 = arena.clone()
            tarr = [np.ascontiguousarray(m_, dtype=np.int64), np.ascontiguousarray(n_, dtype=np.int64),
                    np.ascontiguousarray(np.tile(al, (cnt, 1))), np.asarray(a_p, dtype=np.uint64),
                    np.ascontiguousarray(m_, dtype=np.int64), np.asarray(b_p, dtype=np.uint64),
                    np.ascontiguousarray(m_, dtype=np.int64)]
            tptrs = [x.ctypes.data for x in tarr]
            fn = lambda: lib.lib.mtrsm_grouped(cnt, b"L", b"L", b"N", b"N", *tptrs)
            ms, clk = _timed(torch, fn, args.steps, args.warmup, stream, reset=lambda: arena.copy_(B0))
            value, unit = float(np.sum(m_.astype(np.float64) ** 2 * n_)) / ms / 1e6, "DD-GFLOP/s"
            metric = "batched DD-TRSM GFLOP/s, 5000 LLNN systems n logU[16,256], nrhs U[1,64]"
            cfg = {"workload": "mtrsm_grouped 5000 x L L N N",
                   "launch": "one persistent kernel from a cached CUDA graph, warps pull (instance, 32 right-hand "
                             "sides) items longest first"}
            if o:
                arena.copy_(B0)
                fn()
                torch.cuda.synchronize()
                errs = []
                for t in rng.choice(cnt, 16, replace=False):
                    mm, nn = int(m_[t]), int(n_[t])
                    hA = hb(B0[int(offs[2 * t]):int(offs[2 * t]) + mm * mm]).reshape(mm, mm, 2)
                    want = hb(B0[int(offs[2 * t + 1]):int(offs[2 * t + 1]) + mm * nn]).reshape(nn, mm, 2).copy()
                    o.qtrsm("L", "L", "N", "N", mm, nn, al, hA, mm, want, mm)
                    got = hb(arena[int(offs[2 * t + 1]):int(offs[2 * t + 1]) + mm * nn]).reshape(nn, mm, 2)
                    e = orc.normwise_error(got, want, orc.dd_abs(al) * orc.dd_absmax(want))
                    errs.append(e / (max(20, 8 * mm * mm) * orc.EPS_DD))
                check["max_err_over_tolerance_16_instances"] = float(max(errs))
    else:
        raise SystemExit(f"unknown workload {w}")
    code, msg = lib.last_error()
    if code != 0:
        raise RuntimeError(f"{w}: {code} {msg}")
    launches = lib.lib.mwblas_launch_count() - l0
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64x2 (double-double)", "data": "synthetic (seeded, on device)",
            "config": dict(cfg, l2="operands larger than the 129 MB L2" if w not in ("batched_trsm",) else
                           "arena reset by a device copy between steps"),
            "gpu_launches": int(launches), "clocks": clk, "check": check}
    if roof:
        line["roofline"] = roof
    print(json.dumps(line))
    lib.lib.mwblas_set_stream(None)


if __name__ == "__main__":
    main()
