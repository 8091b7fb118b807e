/* Witness: bench/stencil/jacobi_2d_ref.c (clamp Jacobi sweeps, ping-pong).
 * Returns which buffer (0 or 1) holds the final state. TEST INFRASTRUCTURE ONLY. */
#define main wit_jacobi_unused_main
#include "bench/stencil/jacobi_2d_ref.c"
#undef main
int wit_jacobi(int h, int w, int n_iters, double* buf0, double* buf1) {
    JacobiData d = { h, w, n_iters, buf0, buf1 };
    (void)jacobi_run_once(&d);
    return (n_iters % 2 == 0) ? 0 : 1;
}
