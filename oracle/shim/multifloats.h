/* Clean-room stand-in umbrella header; see multifloats/float64x2.h.
 * TEST INFRASTRUCTURE ONLY (builds the reference sources for parity pinning). */
#pragma once
#include "multifloats/float64x2.h"
