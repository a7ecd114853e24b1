// Complex128 state-vector and density-matrix arithmetic for the oracle
// (TEST INFRASTRUCTURE, never the product): the same operation as
// tfq_oracle.apply_matrix -- a 2^k x 2^k matrix applied to k index bits of a
// 2^nbits vector, optionally only where the control bits match -- written as
// a plain loop so that the oracle can check states of 20-30 qubits and
// density matrices of 14 qubits (a 2^28 vector) in seconds instead of
// minutes.  No fusion, no reordering of the arithmetic beyond one dense
// matrix-vector product per group of 2^k amplitudes, accumulated in double.
//
// The gate semantics (matrices, qubit order, controls) stay in
// tfq_oracle.py, which follows the reference files it cites; this file only
// does the complex128 linear algebra those functions describe.
#include <complex.h>
#include <stdbool.h>
#include <stdint.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

int sv128_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// psi[2^nbits]; m row-major 2^k x 2^k; bits[0] is the index bit of m's most
// significant index bit (bits distinct, none in cmask); only amplitudes whose
// index satisfies (index & cmask) == cval are transformed.
int sv128_apply(cplx* psi, int nbits, const cplx* m, int k, const int* bits,
                uint64_t cmask, uint64_t cval) {
  if (k < 1 || k > 5 || nbits < k || nbits > 40) return -1;
  const int D = 1 << k;
  int sorted[5];
  for (int i = 0; i < k; ++i) sorted[i] = bits[i];
  for (int i = 1; i < k; ++i)
    for (int j = i; j > 0 && sorted[j] < sorted[j - 1]; --j) {
      int t = sorted[j];
      sorted[j] = sorted[j - 1];
      sorted[j - 1] = t;
    }
  uint64_t off[32];
  for (int j = 0; j < D; ++j) {
    uint64_t o = 0;
    for (int i = 0; i < k; ++i)
      if ((j >> (k - 1 - i)) & 1) o |= (uint64_t)1 << bits[i];
    off[j] = o;
  }
  bool diag = true;
  for (int r = 0; r < D && diag; ++r)
    for (int c = 0; c < D; ++c)
      if (r != c && m[r * D + c] != 0) {
        diag = false;
        break;
      }
  const int64_t ngroups = (int64_t)1 << (nbits - k);
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < ngroups; ++g) {
    uint64_t base = (uint64_t)g;
    for (int i = 0; i < k; ++i) {
      const uint64_t low = ((uint64_t)1 << sorted[i]) - 1;
      base = ((base & ~low) << 1) | (base & low);
    }
    if ((base & cmask) != cval) continue;
    if (diag) {
      for (int j = 0; j < D; ++j) psi[base | off[j]] *= m[j * D + j];
      continue;
    }
    cplx v[32], o[32];
    for (int j = 0; j < D; ++j) v[j] = psi[base | off[j]];
    for (int r = 0; r < D; ++r) {
      cplx acc = 0;
      for (int c = 0; c < D; ++c) acc += m[r * D + c] * v[c];
      o[r] = acc;
    }
    for (int j = 0; j < D; ++j) psi[base | off[j]] = o[j];
  }
  return 0;
}

// sum over the vector of conj(a) * b (double accumulation per thread)
void sv128_vdot(const cplx* a, const cplx* b, int64_t len, double* re, double* im) {
  double sr = 0, si = 0;
#pragma omp parallel for reduction(+ : sr, si) schedule(static)
  for (int64_t i = 0; i < len; ++i) {
    const cplx p = conj(a[i]) * b[i];
    sr += creal(p);
    si += cimag(p);
  }
  *re = sr;
  *im = si;
}

// the diagonal of a 2^n x 2^n density matrix stored row-major
void dm128_diagonal(const cplx* rho, int n, double* out) {
  const int64_t dim = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < dim; ++i) out[i] = creal(rho[i * dim + i]);
}
