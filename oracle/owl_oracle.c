/*
 * owl_oracle.c -- CPU oracle for Owl's dense-ndarray conv / pool path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed
 * CPU arm of the benchmark.  The shipped library never links or calls it.
 *
 * Exported entry points keep the names and the argument order of Owl's C
 * stubs (src/owl/core/owl_ndarray_conv_stub.c, owl_ndarray_pool_stub.c), with
 * the OCaml `value` wrappers replaced by plain pointers and longs and the
 * prefix `oracle_` in place of `stub_`.  The algorithms are restated in
 * oracle_impl.h; this file holds the argument plumbing and the padding rules:
 *   forward     : pad = max(0, (stride*(out-1) + k_eff - in) / 2) unless
 *                 padding == 1 (VALID)  -- owl_ndarray_conv_impl.h:288-294,
 *                 :1262-1270, :3145-3150;
 *   backward    : the same expression, always applied (the stubs re-derive
 *                 the padding from the shapes) -- :502-505, :713-716;
 *   non-dilated backward stubs ignore row/col_in_stride -- :491-492.
 *
 * GEMMs go to a BLAS registered at run time (oracle_set_blas), matching Owl's
 * use of cblas_?gemm; without one a plain triple loop is used.
 */

#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  long B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co;
  long sc, sr, sd;  /* strides (cols, rows, depths) */
  long dc, dr, dd;  /* dilation rates ("in strides") */
  long pc, pr, pd;  /* leading padding */
} geom_t;

typedef struct {
  long B, IC, IR, ID, Ch, KC, KR, KD, OC, OR, OD;
  long sc, sr, sd, pc, pr, pd;
} pgeom_t;

/* ---- BLAS registration ------------------------------------------------- */

typedef void (*sgemm32_t)(int, int, int, int, int, int, float, const float *, int,
                          const float *, int, float, float *, int);
typedef void (*dgemm32_t)(int, int, int, int, int, int, double, const double *, int,
                          const double *, int, double, double *, int);
typedef void (*sgemm64_t)(int, int, int, int64_t, int64_t, int64_t, float, const float *,
                          int64_t, const float *, int64_t, float, float *, int64_t);
typedef void (*dgemm64_t)(int, int, int, int64_t, int64_t, int64_t, double, const double *,
                          int64_t, const double *, int64_t, double, double *, int64_t);

/* cblas_cgemm / cblas_zgemm: alpha and beta by pointer, matrices as void *. */
typedef void (*cgemm32_t)(int, int, int, int, int, int, const void *, const void *, int,
                          const void *, int, const void *, void *, int);
typedef void (*cgemm64_t)(int, int, int, int64_t, int64_t, int64_t, const void *, const void *,
                          int64_t, const void *, int64_t, const void *, void *, int64_t);

static void *g_sgemm = 0, *g_dgemm = 0, *g_cgemm = 0, *g_zgemm = 0;
static int g_ilp64 = 0, g_cilp64 = 0;

/* Register cblas_cgemm / cblas_zgemm for the complex kinds (Owl's
 * owl_ndarray_conv_stub.c instantiates the complex stubs with them). */
void oracle_set_blas_complex(void *cgemm, void *zgemm, int ilp64) {
  g_cgemm = cgemm;
  g_zgemm = zgemm;
  g_cilp64 = ilp64;
}

/* Register cblas_sgemm / cblas_dgemm (LP64 when ilp64 == 0, else 64-bit
 * integer interface).  Passing nulls reverts to the built-in loops. */
void oracle_set_blas(void *sgemm, void *dgemm, int ilp64) {
  g_sgemm = sgemm;
  g_dgemm = dgemm;
  g_ilp64 = ilp64;
}

int oracle_has_blas(void) { return g_sgemm != 0 && g_dgemm != 0; }

enum { RowMajor = 101, NoTrans = 111, Trans = 112 };

#define LOOP_GEMM(T)                                                              \
  do {                                                                            \
    for (long i = 0; i < m; ++i)                                                  \
      for (long j = 0; j < n; ++j) {                                              \
        T s = 0;                                                                  \
        for (long p = 0; p < k; ++p) {                                            \
          T av = transA ? A[p * lda + i] : A[i * lda + p];                        \
          T bv = transB ? B[j * ldb + p] : B[p * ldb + j];                        \
          s += av * bv;                                                           \
        }                                                                         \
        C[i * ldc + j] = beta == 0 ? s : beta * C[i * ldc + j] + s;               \
      }                                                                           \
  } while (0)

static void gemm_f32(int transA, int transB, long m, long n, long k, const float *A, long lda,
                     const float *B, long ldb, float beta, float *C, long ldc) {
  if (g_sgemm) {
    if (g_ilp64)
      ((sgemm64_t)g_sgemm)(RowMajor, transA ? Trans : NoTrans, transB ? Trans : NoTrans, m, n, k,
                           1.0f, A, lda, B, ldb, beta, C, ldc);
    else
      ((sgemm32_t)g_sgemm)(RowMajor, transA ? Trans : NoTrans, transB ? Trans : NoTrans, (int)m,
                           (int)n, (int)k, 1.0f, A, (int)lda, B, (int)ldb, beta, C, (int)ldc);
    return;
  }
  LOOP_GEMM(float);
}

static void gemm_f64(int transA, int transB, long m, long n, long k, const double *A, long lda,
                     const double *B, long ldb, double beta, double *C, long ldc) {
  if (g_dgemm) {
    if (g_ilp64)
      ((dgemm64_t)g_dgemm)(RowMajor, transA ? Trans : NoTrans, transB ? Trans : NoTrans, m, n, k,
                           1.0, A, lda, B, ldb, beta, C, ldc);
    else
      ((dgemm32_t)g_dgemm)(RowMajor, transA ? Trans : NoTrans, transB ? Trans : NoTrans, (int)m,
                           (int)n, (int)k, 1.0, A, (int)lda, B, (int)ldb, beta, C, (int)ldc);
    return;
  }
  LOOP_GEMM(double);
}

typedef float _Complex cf32;
typedef double _Complex cf64;

#define CGEMM_VIA(G, CT)                                                                      \
  do {                                                                                        \
    const CT one = 1, bet = beta;                                                             \
    if (g_cilp64)                                                                             \
      ((cgemm64_t)(G))(RowMajor, transA ? Trans : NoTrans, transB ? Trans : NoTrans, m, n, k, \
                       &one, A, lda, B, ldb, &bet, C, ldc);                                   \
    else                                                                                      \
      ((cgemm32_t)(G))(RowMajor, transA ? Trans : NoTrans, transB ? Trans : NoTrans, (int)m,  \
                       (int)n, (int)k, &one, A, (int)lda, B, (int)ldb, &bet, C, (int)ldc);    \
  } while (0)

static void gemm_c32(int transA, int transB, long m, long n, long k, const cf32 *A, long lda,
                     const cf32 *B, long ldb, cf32 beta, cf32 *C, long ldc) {
  if (g_cgemm) {
    CGEMM_VIA(g_cgemm, cf32);
    return;
  }
  LOOP_GEMM(cf32);
}

static void gemm_c64(int transA, int transB, long m, long n, long k, const cf64 *A, long lda,
                     const cf64 *B, long ldb, cf64 beta, cf64 *C, long ldc) {
  if (g_zgemm) {
    CGEMM_VIA(g_zgemm, cf64);
    return;
  }
  LOOP_GEMM(cf64);
}

/* ---- instantiate the algorithms for the four element kinds --------------- */

#define LT(a, b) ((a) < (b))
#define T float
#define SFX f32
#include "oracle_impl.h"
#undef T
#undef SFX

#define T double
#define SFX f64
#include "oracle_impl.h"
#undef T
#undef SFX
#undef LT

/* Owl's complex max pooling starts from -INFINITY, the complex (-inf, 0),
 * whose magnitude is infinite, and compares with CLTF / CLT; the same
 * expressions here (owl_core.h:125, :133). */
#define LT(a, b) \
  ((cabsf(a) < cabsf(b)) || ((cabsf(a) == cabsf(b)) && (cargf(a) < cargf(b))))
#define T cf32
#define SFX c32
#include "oracle_impl.h"
#undef T
#undef SFX
#undef LT

#define LT(a, b) ((cabs(a) < cabs(b)) || ((cabs(a) == cabs(b)) && (carg(a) < carg(b))))
#define T cf64
#define SFX c64
#include "oracle_impl.h"
#undef T
#undef SFX
#undef LT

/* ---- padding rules ----------------------------------------------------- */

static long fwd_pad(long padding, long stride, long out, long keff, long in) {
  if (padding == 1) return 0;
  long p = (stride * (out - 1) + keff - in) / 2; /* C division, as the stubs */
  return p < 0 ? 0 : p;
}

static long bwd_pad(long stride, long out, long keff, long in) {
  long p = (stride * (out - 1) + keff - in) / 2;
  return p < 0 ? 0 : p;
}

static long keff(long k, long rate) { return k + (k - 1) * (rate - 1); }

static geom_t geom3(long B, long IC, long IR, long ID, long Ci, long KC, long KR, long KD, long OC,
                    long OR, long OD, long Co, long sc, long sr, long sd, long dc, long dr,
                    long dd) {
  geom_t g = {B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, sc, sr, sd, dc, dr, dd, 0, 0, 0};
  return g;
}

/* ---- conv entry points (Owl stub argument order) ----------------------- */

#define DEF_CONV_ALL(TY, NAME, SFX2)                                                            \
  /* owl_ndarray_conv_impl.h:246-253 (spatial fwd), dilation fixed at 1 */                      \
  int oracle_##NAME##_ndarray_conv_spatial(                                                     \
      TY *x, TY *w, TY *y, long B, long IC, long IR, long Ci, long KC, long KR, long OC,        \
      long OR, long Co, long sr, long sc, long padding, long rin, long cin) {                   \
    (void)rin; (void)cin;                                                                        \
    geom_t g = geom3(B, IC, IR, 1, Ci, KC, KR, 1, OC, OR, 1, Co, sc, sr, 1, 1, 1, 1);            \
    g.pc = fwd_pad(padding, sc, OC, KC, IC);                                                     \
    g.pr = fwd_pad(padding, sr, OR, KR, IR);                                                     \
    return conv_fwd_##SFX2(&g, x, w, y);                                                         \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:465-472: first argument is dX (written) */                          \
  int oracle_##NAME##_ndarray_conv_spatial_backward_input(                                      \
      TY *dx, TY *w, TY *dy, long B, long IC, long IR, long Ci, long KC, long KR, long OC,       \
      long OR, long Co, long sr, long sc, long rin, long cin) {                                  \
    (void)rin; (void)cin;                                                                        \
    geom_t g = geom3(B, IC, IR, 1, Ci, KC, KR, 1, OC, OR, 1, Co, sc, sr, 1, 1, 1, 1);            \
    g.pc = bwd_pad(sc, OC, KC, IC);                                                              \
    g.pr = bwd_pad(sr, OR, KR, IR);                                                              \
    return conv_bwd_input_##SFX2(&g, dx, w, dy);                                                 \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:675-682: second argument is dW (written) */                         \
  int oracle_##NAME##_ndarray_conv_spatial_backward_kernel(                                     \
      TY *x, TY *dw, TY *dy, long B, long IC, long IR, long Ci, long KC, long KR, long OC,       \
      long OR, long Co, long sr, long sc, long rin, long cin) {                                  \
    (void)rin; (void)cin;                                                                        \
    geom_t g = geom3(B, IC, IR, 1, Ci, KC, KR, 1, OC, OR, 1, Co, sc, sr, 1, 1, 1, 1);            \
    g.pc = bwd_pad(sc, OC, KC, IC);                                                              \
    g.pr = bwd_pad(sr, OR, KR, IR);                                                              \
    return conv_bwd_kernel_##SFX2(&g, x, dw, dy);                                                \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:3097-3150 */                                                        \
  int oracle_##NAME##_ndarray_conv_dilated_spatial_im2col(                                      \
      TY *x, TY *w, TY *y, long B, long IC, long IR, long Ci, long KC, long KR, long OC,        \
      long OR, long Co, long sr, long sc, long padding, long rin, long cin) {                   \
    geom_t g = geom3(B, IC, IR, 1, Ci, KC, KR, 1, OC, OR, 1, Co, sc, sr, 1, cin, rin, 1);        \
    g.pc = fwd_pad(padding, sc, OC, keff(KC, cin), IC);                                          \
    g.pr = fwd_pad(padding, sr, OR, keff(KR, rin), IR);                                          \
    return conv_fwd_##SFX2(&g, x, w, y);                                                         \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:3317-3350 */                                                        \
  int oracle_##NAME##_ndarray_conv_dilated_spatial_backward_input_im2col(                       \
      TY *dx, TY *w, TY *dy, long B, long IC, long IR, long Ci, long KC, long KR, long OC,       \
      long OR, long Co, long sr, long sc, long rin, long cin) {                                  \
    geom_t g = geom3(B, IC, IR, 1, Ci, KC, KR, 1, OC, OR, 1, Co, sc, sr, 1, cin, rin, 1);        \
    g.pc = bwd_pad(sc, OC, keff(KC, cin), IC);                                                   \
    g.pr = bwd_pad(sr, OR, keff(KR, rin), IR);                                                   \
    return conv_bwd_input_##SFX2(&g, dx, w, dy);                                                 \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:3203-3240 */                                                        \
  int oracle_##NAME##_ndarray_conv_dilated_spatial_backward_kernel_im2col(                      \
      TY *x, TY *dw, TY *dy, long B, long IC, long IR, long Ci, long KC, long KR, long OC,       \
      long OR, long Co, long sr, long sc, long rin, long cin) {                                  \
    geom_t g = geom3(B, IC, IR, 1, Ci, KC, KR, 1, OC, OR, 1, Co, sc, sr, 1, cin, rin, 1);        \
    g.pc = bwd_pad(sc, OC, keff(KC, cin), IC);                                                   \
    g.pr = bwd_pad(sr, OR, keff(KR, rin), IR);                                                   \
    return conv_bwd_kernel_##SFX2(&g, x, dw, dy);                                                \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:1211-1219 */                                                        \
  int oracle_##NAME##_ndarray_conv_cuboid_im2col(                                               \
      TY *x, TY *w, TY *y, long B, long IC, long IR, long ID, long Ci, long KC, long KR,        \
      long KD, long OC, long OR, long OD, long Co, long sd, long sr, long sc, long padding) {    \
    geom_t g = geom3(B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, sc, sr, sd, 1, 1, 1);        \
    g.pc = fwd_pad(padding, sc, OC, KC, IC);                                                     \
    g.pr = fwd_pad(padding, sr, OR, KR, IR);                                                     \
    g.pd = fwd_pad(padding, sd, OD, KD, ID);                                                     \
    return conv_fwd_##SFX2(&g, x, w, y);                                                         \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:1456-1463 */                                                        \
  int oracle_##NAME##_ndarray_conv_cuboid_backward_input_im2col(                                \
      TY *dx, TY *w, TY *dy, long B, long IC, long IR, long ID, long Ci, long KC, long KR,       \
      long KD, long OC, long OR, long OD, long Co, long sd, long sr, long sc) {                  \
    geom_t g = geom3(B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, sc, sr, sd, 1, 1, 1);        \
    g.pc = bwd_pad(sc, OC, KC, IC);                                                              \
    g.pr = bwd_pad(sr, OR, KR, IR);                                                              \
    g.pd = bwd_pad(sd, OD, KD, ID);                                                              \
    return conv_bwd_input_##SFX2(&g, dx, w, dy);                                                 \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:1331-1338 */                                                        \
  int oracle_##NAME##_ndarray_conv_cuboid_backward_kernel_im2col(                               \
      TY *x, TY *dw, TY *dy, long B, long IC, long IR, long ID, long Ci, long KC, long KR,       \
      long KD, long OC, long OR, long OD, long Co, long sd, long sr, long sc) {                  \
    geom_t g = geom3(B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, sc, sr, sd, 1, 1, 1);        \
    g.pc = bwd_pad(sc, OC, KC, IC);                                                              \
    g.pr = bwd_pad(sr, OR, KR, IR);                                                              \
    g.pd = bwd_pad(sd, OD, KD, ID);                                                              \
    return conv_bwd_kernel_##SFX2(&g, x, dw, dy);                                                \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:3417-3426 */                                                        \
  int oracle_##NAME##_ndarray_conv_dilated_cuboid_im2col(                                       \
      TY *x, TY *w, TY *y, long B, long IC, long IR, long ID, long Ci, long KC, long KR,        \
      long KD, long OC, long OR, long OD, long Co, long sd, long sr, long sc, long din,         \
      long rin, long cin, long padding) {                                                        \
    geom_t g = geom3(B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, sc, sr, sd, cin, rin, din);  \
    g.pc = fwd_pad(padding, sc, OC, keff(KC, cin), IC);                                          \
    g.pr = fwd_pad(padding, sr, OR, keff(KR, rin), IR);                                          \
    g.pd = fwd_pad(padding, sd, OD, keff(KD, din), ID);                                          \
    return conv_fwd_##SFX2(&g, x, w, y);                                                         \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:3678-3686 */                                                        \
  int oracle_##NAME##_ndarray_conv_dilated_cuboid_backward_input_im2col(                        \
      TY *dx, TY *w, TY *dy, long B, long IC, long IR, long ID, long Ci, long KC, long KR,       \
      long KD, long OC, long OR, long OD, long Co, long sd, long sr, long sc, long din,          \
      long rin, long cin) {                                                                      \
    geom_t g = geom3(B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, sc, sr, sd, cin, rin, din);  \
    g.pc = bwd_pad(sc, OC, keff(KC, cin), IC);                                                   \
    g.pr = bwd_pad(sr, OR, keff(KR, rin), IR);                                                   \
    g.pd = bwd_pad(sd, OD, keff(KD, din), ID);                                                   \
    return conv_bwd_input_##SFX2(&g, dx, w, dy);                                                 \
  }                                                                                              \
  /* owl_ndarray_conv_impl.h:3545-3553 */                                                        \
  int oracle_##NAME##_ndarray_conv_dilated_cuboid_backward_kernel_im2col(                       \
      TY *x, TY *dw, TY *dy, long B, long IC, long IR, long ID, long Ci, long KC, long KR,       \
      long KD, long OC, long OR, long OD, long Co, long sd, long sr, long sc, long din,          \
      long rin, long cin) {                                                                      \
    geom_t g = geom3(B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co, sc, sr, sd, cin, rin, din);  \
    g.pc = bwd_pad(sc, OC, keff(KC, cin), IC);                                                   \
    g.pr = bwd_pad(sr, OR, keff(KR, rin), IR);                                                   \
    g.pd = bwd_pad(sd, OD, keff(KD, din), ID);                                                   \
    return conv_bwd_kernel_##SFX2(&g, x, dw, dy);                                                \
  }

DEF_CONV_ALL(float, float32, f32)
DEF_CONV_ALL(double, float64, f64)
DEF_CONV_ALL(cf32, complex32, c32)
DEF_CONV_ALL(cf64, complex64, c64)

/* ---- pool entry points (Owl stub argument order) ----------------------- */

static pgeom_t pgeom(long B, long IC, long IR, long ID, long Ch, long KC, long KR, long KD,
                     long OC, long OR, long OD, long sc, long sr, long sd) {
  pgeom_t g = {B, IC, IR, ID, Ch, KC, KR, KD, OC, OR, OD, sc, sr, sd, 0, 0, 0};
  return g;
}

#define DEF_POOL_ALL(TY, NAME, SFX2, KIND, MODE)                                                 \
  /* owl_ndarray_pool_impl.h:9-15 (fwd), padding flag as :43-49 */                              \
  int oracle_##NAME##_ndarray_##KIND##_spatial(                                                 \
      TY *x, TY *y, long B, long IC, long IR, long Ch, long KC, long KR, long OC, long OR,      \
      long sr, long sc, long padding, long rin, long cin) {                                      \
    (void)rin; (void)cin;                                                                        \
    pgeom_t g = pgeom(B, IC, IR, 1, Ch, KC, KR, 1, OC, OR, 1, sc, sr, 1);                        \
    g.pr = fwd_pad(padding, sr, OR, KR, IR);                                                     \
    g.pc = fwd_pad(padding, sc, OC, KC, IC);                                                     \
    pool_fwd_##SFX2(&g, x, y, 0, MODE);                                                          \
    return 0;                                                                                    \
  }                                                                                              \
  /* owl_ndarray_pool_impl.h:102-108: explicit pads, negatives clipped (:136-137) */            \
  int oracle_##NAME##_ndarray_##KIND##_spatial_backward(                                        \
      TY *x, TY *dy, TY *dx, long B, long IC, long IR, long Ch, long KC, long KR, long OC,      \
      long OR, long sr, long sc, long pad_rows, long pad_cols) {                                 \
    pgeom_t g = pgeom(B, IC, IR, 1, Ch, KC, KR, 1, OC, OR, 1, sc, sr, 1);                        \
    g.pr = pad_rows < 0 ? 0 : pad_rows;                                                          \
    g.pc = pad_cols < 0 ? 0 : pad_cols;                                                          \
    pool_bwd_##SFX2(&g, x, dy, dx, MODE);                                                        \
    return 0;                                                                                    \
  }                                                                                              \
  /* owl_ndarray_pool_impl.h:212-219 */                                                          \
  int oracle_##NAME##_ndarray_##KIND##_cuboid(                                                  \
      TY *x, TY *y, long B, long IC, long IR, long ID, long Ch, long KC, long KR, long KD,      \
      long OC, long OR, long OD, long sd, long sr, long sc, long padding) {                      \
    pgeom_t g = pgeom(B, IC, IR, ID, Ch, KC, KR, KD, OC, OR, OD, sc, sr, sd);                    \
    g.pc = fwd_pad(padding, sc, OC, KC, IC);                                                     \
    g.pr = fwd_pad(padding, sr, OR, KR, IR);                                                     \
    g.pd = fwd_pad(padding, sd, OD, KD, ID);                                                     \
    pool_fwd_##SFX2(&g, x, y, 0, MODE);                                                          \
    return 0;                                                                                    \
  }                                                                                              \
  /* owl_ndarray_pool_impl.h:324-331: strides arrive col, row, dpt */                           \
  int oracle_##NAME##_ndarray_##KIND##_cuboid_backward(                                         \
      TY *x, TY *dy, TY *dx, long B, long IC, long IR, long ID, long Ch, long KC, long KR,      \
      long KD, long OC, long OR, long OD, long sc, long sr, long sd, long padding) {             \
    pgeom_t g = pgeom(B, IC, IR, ID, Ch, KC, KR, KD, OC, OR, OD, sc, sr, sd);                    \
    g.pc = fwd_pad(padding, sc, OC, KC, IC);                                                     \
    g.pr = fwd_pad(padding, sr, OR, KR, IR);                                                     \
    g.pd = fwd_pad(padding, sd, OD, KD, ID);                                                     \
    pool_bwd_##SFX2(&g, x, dy, dx, MODE);                                                        \
    return 0;                                                                                    \
  }

DEF_POOL_ALL(float, float32, f32, maxpool, 0)
DEF_POOL_ALL(float, float32, f32, avgpool, 1)
DEF_POOL_ALL(double, float64, f64, maxpool, 0)
DEF_POOL_ALL(double, float64, f64, avgpool, 1)
DEF_POOL_ALL(cf32, complex32, c32, maxpool, 0)
DEF_POOL_ALL(cf32, complex32, c32, avgpool, 1)
DEF_POOL_ALL(cf64, complex64, c64, maxpool, 0)
DEF_POOL_ALL(cf64, complex64, c64, avgpool, 1)

/* owl_ndarray_pool_impl.h:459-465: max value plus int64 flat argmax */
#define DEF_ARG(TY, NAME, SFX2)                                                                 \
  int oracle_##NAME##_ndarray_maxpool_spatial_arg(                                              \
      TY *x, TY *y, int64_t *arg, long B, long IC, long IR, long Ch, long KC, long KR,          \
      long OC, long OR, long sr, long sc, long pad_rows, long pad_cols) {                        \
    pgeom_t g = pgeom(B, IC, IR, 1, Ch, KC, KR, 1, OC, OR, 1, sc, sr, 1);                        \
    g.pr = pad_rows < 0 ? 0 : pad_rows;                                                          \
    g.pc = pad_cols < 0 ? 0 : pad_cols;                                                          \
    pool_fwd_##SFX2(&g, x, y, arg, 0);                                                           \
    return 0;                                                                                    \
  }
DEF_ARG(float, float32, f32)
DEF_ARG(double, float64, f64)
DEF_ARG(cf32, complex32, c32)
DEF_ARG(cf64, complex64, c64)

/* ---- nearest-neighbour 2-D upsampling ----------------------------------
 * Backward: owl_ndarray_upsampling_impl.h:9-58 -- zero dX, then for every
 * output position (b, c, r) in order, dX at (min(c / sc, IC - 1),
 * min(r / sr, IR - 1)) += dY.  Forward: Owl's upsampling2d is
 * `repeat x [|1; sc; sr; 1|]` (owl_dense_ndarray_generic.ml:8223-8233), so
 * y[b][c][r] = x[b][c / sc][r / sr] over the repeated extents. */
#define DEF_UP(TY, NAME)                                                                        \
  int oracle_##NAME##_ndarray_upsampling_spatial_backward(                                      \
      TY *dx, const TY *dy, long B, long IC, long IR, long Ch, long OC, long OR, long sc,       \
      long sr) {                                                                                 \
    memset(dx, 0, sizeof(TY) * (size_t)(B * IC * IR * Ch));                                     \
    for (long b = 0; b < B; ++b)                                                                 \
      for (long c = 0; c < OC; ++c) {                                                            \
        const long ic = c / sc < IC - 1 ? c / sc : IC - 1;                                       \
        for (long r = 0; r < OR; ++r) {                                                          \
          const long ir = r / sr < IR - 1 ? r / sr : IR - 1;                                    \
          TY *d = dx + ((b * IC + ic) * IR + ir) * Ch;                                           \
          const TY *s = dy + ((b * OC + c) * OR + r) * Ch;                                       \
          for (long i = 0; i < Ch; ++i) d[i] += s[i];                                            \
        }                                                                                        \
      }                                                                                          \
    return 0;                                                                                    \
  }                                                                                              \
  int oracle_##NAME##_ndarray_upsampling_spatial(                                               \
      const TY *x, TY *y, long B, long IC, long IR, long Ch, long OC, long OR, long sc,         \
      long sr) {                                                                                 \
    if (OC != IC * sc || OR != IR * sr) return -1;                                               \
    for (long b = 0; b < B; ++b)                                                                 \
      for (long c = 0; c < OC; ++c)                                                              \
        for (long r = 0; r < OR; ++r)                                                            \
          memcpy(y + ((b * OC + c) * OR + r) * Ch, x + ((b * IC + c / sc) * IR + r / sr) * Ch,   \
                 sizeof(TY) * (size_t)Ch);                                                       \
    return 0;                                                                                    \
  }
DEF_UP(float, float32)
DEF_UP(double, float64)
DEF_UP(cf32, complex32)
DEF_UP(cf64, complex64)
