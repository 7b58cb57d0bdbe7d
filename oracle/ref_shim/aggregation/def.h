/*
 * Project-written stand-in for the `aggregation/def.h` header of the
 * reference's `aggregation` git submodule, which is not vendored (its commit
 * is not pinned anywhere in the reference tree).  It declares only what the
 * reference's hot-path translation units need in order to compile:
 *   - the EMPTY / NULLPNTR sentinels used by spilu0.cpp;
 *   - opaque CSC / CSR / Dense structs named in sparse_blas_lib.h signatures
 *     (no hot-path function dereferences them).
 * Test infrastructure only: used when compiling the reference into the
 * oracle's reference library, never by the product.
 */
#ifndef GBSYM_REF_SHIM_AGGREGATION_DEF_H
#define GBSYM_REF_SHIM_AGGREGATION_DEF_H
#include <cassert>
#include <cmath>
#include <cstddef>
#include <algorithm>

#define EMPTY (-1)
#define NULLPNTR nullptr

namespace sym_lib {
 struct CSC { int m, n, nnz, stype; bool is_pattern, pre_alloc; int *p, *i; double *x; };
 struct CSR { int m, n, nnz, stype; bool is_pattern, pre_alloc; int *p, *i; double *x; };
 struct Dense { int row, col, lda; double *a; };
}
#endif
