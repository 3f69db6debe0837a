// Host-side harness for epblas-parallel_gb300/csrc/xfloat.cuh and xword.cuh
// (the integer extended-float arithmetic of the CRT reconstruction, as
// __int128 and as 32-bit words), compiled with g++ by tests/test_xfloat.py so
// the device code's logic is checked on the CPU.
#include "../epblas-parallel_gb300/csrc/xfloat.cuh"

extern "C" {

void xf_roundtrip(double hi, double lo, double *oh, double *ol)
{
    xfp::XF x = xfp::xf_from_dd(hi, lo);
    xfp::xf_to_dd(x, *oh, *ol);
}

void xf_mul_dd(double ah, double al, double bh, double bl, double *oh, double *ol)
{
    xfp::xf_to_dd(xfp::xf_mul(xfp::xf_from_dd(ah, al), xfp::xf_from_dd(bh, bl)), *oh, *ol);
}

void xf_add_dd(double ah, double al, double bh, double bl, double *oh, double *ol)
{
    xfp::xf_to_dd(xfp::xf_add(xfp::xf_from_dd(ah, al), xfp::xf_from_dd(bh, bl)), *oh, *ol);
}

// alpha * a + beta * c, the reconstruction's update
void xf_axpby(double alh, double all, double ah, double al, double beh, double bel, double ch, double cl, double *oh,
              double *ol)
{
    xfp::XF v = xfp::xf_mul(xfp::xf_from_dd(alh, all), xfp::xf_from_dd(ah, al));
    xfp::XF w = xfp::xf_mul(xfp::xf_from_dd(beh, bel), xfp::xf_from_dd(ch, cl));
    xfp::xf_to_dd(xfp::xf_add(v, w), *oh, *ol);
}

}

// CRT reconstruction in fractional fixed point (csrc/crt.cuh): residues c[l]
// of X modulo p[l] -> X * 2^-S2 as a double-double.
#include "../epblas-parallel_gb300/csrc/crt.cuh"

extern "C" void crt_frac(int n, const int *p, const int *c, int S2, double *oh, double *ol)
{
    uint32_t F[40][crt::kFLPad];
    xfp::XF Mx;
    crt::constants(p, n, F, Mx);
    crt::Frac acc;
    acc.reset();
    for (int l = 0; l < n; ++l) acc.add(F[l], (uint32_t)c[l]);
    xfp::xf_to_dd(acc.finish(Mx, S2), *oh, *ol);
}

// The same operations on the 32-bit-word extended floats (csrc/xword.cuh).
extern "C" {

void xw_roundtrip(double hi, double lo, double *oh, double *ol)
{
    xw::to_dd(xw::from_dd(hi, lo), *oh, *ol);
}

void xw_mul_dd(double ah, double al, double bh, double bl, double *oh, double *ol)
{
    xw::to_dd(xw::mul(xw::from_dd(ah, al), xw::from_dd(bh, bl)), *oh, *ol);
}

void xw_add_dd(double ah, double al, double bh, double bl, double *oh, double *ol)
{
    xw::to_dd(xw::add(xw::from_dd(ah, al), xw::from_dd(bh, bl)), *oh, *ol);
}

void xw_axpby(double alh, double all, double ah, double al, double beh, double bel, double ch, double cl, double *oh,
              double *ol)
{
    xw::XW v = xw::mul(xw::from_dd(alh, all), xw::from_dd(ah, al));
    xw::XW w = xw::mul(xw::from_dd(beh, bel), xw::from_dd(ch, cl));
    xw::to_dd(xw::add(v, w), *oh, *ol);
}

void crt_frac_xw(int n, const int *p, const int *c, int S2, double *oh, double *ol)
{
    uint32_t F[40][crt::kFLPad];
    xfp::XF Mx;
    crt::constants(p, n, F, Mx);
    crt::Frac acc;
    acc.reset();
    for (int l = 0; l < n; ++l) acc.add(F[l], (uint32_t)c[l]);
    xw::to_dd(acc.finish_xw(crt::to_xw(Mx), S2), *oh, *ol);
}

}
