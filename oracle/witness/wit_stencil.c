/* Witness: bench/stencil/stencil_ref.c (one clamp Laplacian sweep).
 * TEST INFRASTRUCTURE ONLY. */
#define main wit_stencil_unused_main
#include "bench/stencil/stencil_ref.c"
#undef main
void wit_laplacian(int h, int w, double* in, double* out) {
    StencilData d = { h, w, in, out };
    (void)stencil_run_once(&d);
}
