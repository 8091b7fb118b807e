/* Witness: bench/weighted_histogram/weighted_histogram_ref.c (atomic OpenMP
 * histogram of bucket (i*bins)/n, weight 3i+1). TEST INFRASTRUCTURE ONLY. */
#define main wit_whist_unused_main
#include "bench/weighted_histogram/weighted_histogram_ref.c"
#undef main
void wit_whist(int64_t n, int64_t bins, int64_t* hist) {
    WHData d = { n, bins, hist };
    (void)wh_run_once(&d);
}
