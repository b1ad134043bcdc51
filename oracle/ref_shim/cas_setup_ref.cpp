// cas_setup_ref.cpp - the reference's CasSetup (shaders/ffx_cas.h:375-394),
// compiled for the CPU from the vendored header as source/taa.hpp:15-19 does
// (A_CPU), to pin the oracle's restatement.  Test infrastructure.
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
// the including translation unit provides the C math library, as gvk does for taa.hpp
#define A_CPU 1
#include "ffx_a.h"
#include "ffx_cas.h"

extern "C" void ref_cas_setup(float sharpness, float in_w, float in_h, float out_w, float out_h, uint32_t* c0,
                              uint32_t* c1) {
    varAU4(const0);
    varAU4(const1);
    CasSetup(const0, const1, sharpness, in_w, in_h, out_w, out_h);
    for (int i = 0; i < 4; ++i) {
        c0[i] = const0[i];
        c1[i] = const1[i];
    }
}
