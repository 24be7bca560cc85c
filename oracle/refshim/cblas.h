/*
 * Minimal CBLAS shim used only to compile the unmodified reference sources
 * (test infrastructure, never part of the product).
 *
 * The reference includes <cblas.h> (src/tensor.cpp:24) and calls
 * cblas_cgemm / cblas_cgemv / cblas_cdotu_sub (src/tensor.cpp:973,995,1018,
 * 1039). No system OpenBLAS is installed here, but scipy bundles OpenBLAS
 * 0.3.x with an LP64 CBLAS interface whose symbols carry a "scipy_" prefix.
 * This header declares those symbols and forwards the reference's calls.
 *
 * When QFLEX_REF_GEMM_LOG names a file, every complex GEMM/GEMV/DOT shape is
 * appended to it as "<kind> m n k", so the engine's planned shape list can be
 * compared against the reference's actual BLAS calls.
 */
#ifndef QFLEX_REFSHIM_CBLAS_H
#define QFLEX_REFSHIM_CBLAS_H

#include <cstdio>
#include <cstdlib>

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE {
  CblasNoTrans = 111,
  CblasTrans = 112,
  CblasConjTrans = 113,
  CblasConjNoTrans = 114
};
typedef struct {
  float real;
  float imag;
} openblas_complex_float;

extern "C" {
void scipy_cblas_cgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE,
                       enum CBLAS_TRANSPOSE, int m, int n, int k,
                       const void* alpha, const void* a, int lda,
                       const void* b, int ldb, const void* beta, void* c,
                       int ldc);
void scipy_cblas_cgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, int m, int n,
                       const void* alpha, const void* a, int lda,
                       const void* x, int incx, const void* beta, void* y,
                       int incy);
void scipy_cblas_cdotu_sub(int n, const void* x, int incx, const void* y,
                           int incy, void* ret);
void scipy_openblas_set_num_threads(int);
}

namespace qflex_refshim {
inline void log_shape(const char* kind, long m, long n, long k) {
  static FILE* f = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    if (const char* p = std::getenv("QFLEX_REF_GEMM_LOG")) f = std::fopen(p, "w");
  }
  if (f) std::fprintf(f, "%s %ld %ld %ld\n", kind, m, n, k);
}
}  // namespace qflex_refshim

inline void cblas_cgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta,
                        enum CBLAS_TRANSPOSE tb, long m, long n, long k,
                        const void* alpha, const void* a, long lda,
                        const void* b, long ldb, const void* beta, void* c,
                        long ldc) {
  qflex_refshim::log_shape("MM", m, n, k);
  scipy_cblas_cgemm(o, ta, tb, (int)m, (int)n, (int)k, alpha, a, (int)lda, b,
                    (int)ldb, beta, c, (int)ldc);
}

inline void cblas_cgemv(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE t, long m,
                        long n, const void* alpha, const void* a, long lda,
                        const void* x, long incx, const void* beta, void* y,
                        long incy) {
  // Row-major NoTrans is the reference's Mv (m rows, k = n); Trans is its vM
  // (rows = k, columns = n).
  if (t == CblasNoTrans)
    qflex_refshim::log_shape("Mv", m, 1, n);
  else
    qflex_refshim::log_shape("vM", 1, n, m);
  scipy_cblas_cgemv(o, t, (int)m, (int)n, alpha, a, (int)lda, x, (int)incx,
                    beta, y, (int)incy);
}

inline void cblas_cdotu_sub(long n, const void* x, long incx, const void* y,
                            long incy, void* ret) {
  qflex_refshim::log_shape("vv", 1, 1, n);
  scipy_cblas_cdotu_sub((int)n, x, (int)incx, y, (int)incy, ret);
}

#endif
