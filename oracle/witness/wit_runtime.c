/* Witness: the reference runtime header's stable LSD radix sort_indices
 * (runtime/hydrangea_runtime.h:386-456), compiled unmodified against the
 * project's scalar SIMDe shim. TEST INFRASTRUCTURE ONLY. */
#include <stdint.h>
#include <string.h>
#include "runtime/hydrangea_runtime.h"

/* getenv_int / getenv_string, which the header declares, come from the
 * reference's runtime/hyd_write_csv.c (wit_csv.c). */

void wit_sort_indices(const int64_t* keys, int64_t n, int64_t* perm) {
    hyd_tuple_t shape;
    shape.ndims = 1;
    shape.elems[0] = n;
    hyd_array_t* k = hyd_array_alloc(shape);
    memcpy(k->data, keys, (size_t)n * sizeof(int64_t));
    hyd_array_t* p = hyd_sort_indices(k);
    memcpy(perm, p->data, (size_t)n * sizeof(int64_t));
    hyd_array_free(p);
    hyd_array_free(k);
}

/* nd <-> flat helpers (runtime/hydrangea_runtime.h:365-384) */
int64_t wit_nd_to_flat2(int64_t i, int64_t j, int64_t h, int64_t w) {
    hyd_tuple_t nd, shape;
    nd.ndims = 2; nd.elems[0] = i; nd.elems[1] = j;
    shape.ndims = 2; shape.elems[0] = h; shape.elems[1] = w;
    return hyd_nd_to_flat(nd, shape);
}
