// Column tridiagonal elimination in the operation order of LAPACK dgtsv
// (Gaussian elimination with partial pivoting, one right-hand side), the
// routine the reference calls (veros/core/operators.py:75). Every product,
// difference and quotient is an explicitly rounded intrinsic, so the compiler
// cannot contract them into FMAs and the results match dgtsv's IEEE
// arithmetic operation for operation.
//
// A column is the system of rows k = ks..Z-1. A row source provides
//   a(k)  entry left of the diagonal in row k   (used for k > ks)
//   b(k)  diagonal (edge-substituted at ks)
//   c(k)  entry right of the diagonal (k < Z-1)
//   d(k)  right-hand side (edge-substituted at ks)
//
// Fast path (callers inline it in their own k loops): no row interchange,
// which dgtsv also takes whenever |d_k| >= |a_{k+1}|. If some row would need
// an interchange, the caller runs dgtsv_slow_solve, which re-derives each
// row's final factors by replaying the elimination from ks (O(n^2) work, O(1)
// storage beyond the solution).
#pragma once

#include <cuda_runtime.h>

namespace vg {

__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

struct RowFactors {
  double d, du, du2, b;
};

// Final factors of row kt after the elimination steps ks..kt (row kt as pivot row).
template <class Src>
__device__ RowFactors dgtsv_final_row(const Src &s, int ks, int Z, int kt) {
  double cd = s.b(ks), cdu = ks < Z - 1 ? s.c(ks) : 0.0, cb = s.d(ks);
  for (int k = ks;; ++k) {
    if (k == Z - 1) return RowFactors{cd, 0.0, 0.0, cb};
    const double dl = s.a(k + 1);
    const double dn = s.b(k + 1);
    const double dun = (k + 1 < Z - 1) ? s.c(k + 1) : 0.0;
    const double bn = s.d(k + 1);
    RowFactors fin;
    double nd, ndu, nb;
    if (fabs(cd) >= fabs(dl)) {
      const double fact = rdiv(dl, cd);
      fin = RowFactors{cd, cdu, 0.0, cb};
      nd = rsub(dn, rmul(fact, cdu));
      ndu = dun;
      nb = rsub(bn, rmul(fact, cb));
    } else {
      const double fact = rdiv(cd, dl);
      const bool last = k == Z - 2;
      fin = RowFactors{dl, dn, last ? 0.0 : dun, bn};
      nd = rsub(cdu, rmul(fact, dn));
      ndu = last ? dun : -rmul(fact, dun);
      nb = rsub(cb, rmul(fact, bn));
    }
    if (k == kt) return fin;
    cd = nd;
    cdu = ndu;
    cb = nb;
  }
}

// Solution of one column with interchanges; x(k) goes to xs[k * xstride].
template <class Src>
__device__ void dgtsv_slow_solve(const Src &s, int ks, int Z, double *xs, int xstride) {
  double x1 = 0.0, x2 = 0.0;
  for (int kt = Z - 1; kt >= ks; --kt) {
    const RowFactors f = dgtsv_final_row(s, ks, Z, kt);
    double x;
    if (kt == Z - 1)
      x = rdiv(f.b, f.d);
    else if (kt == Z - 2)
      x = rdiv(rsub(f.b, rmul(f.du, x1)), f.d);
    else
      x = rdiv(rsub(rsub(f.b, rmul(f.du, x1)), rmul(f.du2, x2)), f.d);
    xs[(size_t)kt * xstride] = x;
    x2 = x1;
    x1 = x;
  }
}

}  // namespace vg
