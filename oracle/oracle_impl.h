/*
 * CPU oracle for the Owl dense-ndarray convolution / pooling path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links or calls
 * this code; only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it, and only as the checker (or as the timed CPU arm).
 *
 * This header is instantiated four times by owl_oracle.c: T=float (Owl's S
 * module), T=double (D), T=float _Complex (C) and T=double _Complex (Z).
 * LT(a, b) is the ordering max pooling uses: `<` for the reals, magnitude
 * then argument for the complex kinds (CLTF / CLT, owl_core.h:125, :133).  Every function
 * restates the algorithm of the Owl C stub named in its comment:
 *   conv  : im2col followed by one GEMM per block of output pixels, the
 *           strategy of src/owl/core/owl_ndarray_conv_impl.h:296-338 (2-D),
 *           :1211-1323 (3-D) and :3097-3195 (dilated);
 *   pool  : the exact scan order, comparison and accumulation type of
 *           src/owl/core/owl_ndarray_pool_impl.h:9-543, because pooling
 *           results must match bit for bit.
 */

#if !defined(T) || !defined(SFX) || !defined(LT)
#error "instantiate with T, SFX and LT defined"
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* im2col row for output pixel index `m` (flat over b, oc, or, od), columns
 * ordered ((kc*KR + kr)*KD + kd)*Ci + ci, zero where the tap falls in the
 * padding.  Mirrors the fill loops of owl_ndarray_conv_impl.h:1280-1310 and
 * :3160-3180 (dilated taps advance by the in-stride). */
static void FN(im2col_row_)(const geom_t *g, const T *x, long m, T *row) {
  long od = m % g->OD;
  long t = m / g->OD;
  long orr = t % g->OR;
  t /= g->OR;
  long oc = t % g->OC;
  long b = t / g->OC;
  long c0 = oc * g->sc - g->pc, r0 = orr * g->sr - g->pr, d0 = od * g->sd - g->pd;
  const T *xb = x + b * g->IC * g->IR * g->ID * g->Ci;
  long cnt = 0;
  for (long kc = 0; kc < g->KC; ++kc) {
    long a = c0 + kc * g->dc;
    for (long kr = 0; kr < g->KR; ++kr) {
      long bb = r0 + kr * g->dr;
      for (long kd = 0; kd < g->KD; ++kd) {
        long c = d0 + kd * g->dd;
        int inb = a >= 0 && a < g->IC && bb >= 0 && bb < g->IR && c >= 0 && c < g->ID;
        if (inb) {
          const T *src = xb + ((a * g->IR + bb) * g->ID + c) * g->Ci;
          memcpy(row + cnt, src, sizeof(T) * g->Ci);
        } else {
          memset(row + cnt, 0, sizeof(T) * g->Ci);
        }
        cnt += g->Ci;
      }
    }
  }
}

/* col2im: add one row of the column matrix back into dX, in the same
 * element order as owl_ndarray_conv_impl.h:1520-1545 (`input_ptr[...] +=`). */
static void FN(col2im_row_add_)(const geom_t *g, T *dx, long m, const T *row) {
  long od = m % g->OD;
  long t = m / g->OD;
  long orr = t % g->OR;
  t /= g->OR;
  long oc = t % g->OC;
  long b = t / g->OC;
  long c0 = oc * g->sc - g->pc, r0 = orr * g->sr - g->pr, d0 = od * g->sd - g->pd;
  T *xb = dx + b * g->IC * g->IR * g->ID * g->Ci;
  long cnt = 0;
  for (long kc = 0; kc < g->KC; ++kc) {
    long a = c0 + kc * g->dc;
    for (long kr = 0; kr < g->KR; ++kr) {
      long bb = r0 + kr * g->dr;
      for (long kd = 0; kd < g->KD; ++kd) {
        long c = d0 + kd * g->dd;
        if (a >= 0 && a < g->IC && bb >= 0 && bb < g->IR && c >= 0 && c < g->ID) {
          T *dst = xb + ((a * g->IR + bb) * g->ID + c) * g->Ci;
          for (long h = 0; h < g->Ci; ++h) dst[h] += row[cnt + h];
        }
        cnt += g->Ci;
      }
    }
  }
}

static long FN(block_rows_)(const geom_t *g) {
  long K = g->KC * g->KR * g->KD * g->Ci;
  long M = g->B * g->OC * g->OR * g->OD;
  long mb = (1L << 25) / (K > 0 ? K : 1); /* ~128 MB of float column matrix */
  if (mb < 1) mb = 1;
  if (mb > M) mb = M;
  return mb;
}

/* Y = X (*) W.  Restates the im2col + GEMM forward of
 * owl_ndarray_conv_impl.h:296-338 / :1262-1320 / :3145-3190, blocked over
 * output pixels the way the GEBP path (:340-446) blocks its m dimension. */
static int FN(conv_fwd_)(const geom_t *g, const T *x, const T *w, T *y) {
  long K = g->KC * g->KR * g->KD * g->Ci;
  long M = g->B * g->OC * g->OR * g->OD;
  memset(y, 0, sizeof(T) * M * g->Co);
  if (M == 0 || K == 0 || g->Co == 0) return 0;
  long mb = FN(block_rows_)(g);
  T *col = (T *)malloc(sizeof(T) * mb * K);
  if (!col) return -1;
  for (long m0 = 0; m0 < M; m0 += mb) {
    long rows = (M - m0 < mb) ? M - m0 : mb;
    for (long i = 0; i < rows; ++i) FN(im2col_row_)(g, x, m0 + i, col + i * K);
    FN(gemm_)(0, 0, rows, g->Co, K, col, K, w, g->Co, (T)0, y + m0 * g->Co, g->Co);
  }
  free(col);
  return 0;
}

/* dX = col2im(dY * W^T).  Restates owl_ndarray_conv_impl.h:510-560 and
 * :1480-1550 (GEMM with the kernel transposed, then scatter-add). */
static int FN(conv_bwd_input_)(const geom_t *g, T *dx, const T *w, const T *dy) {
  long K = g->KC * g->KR * g->KD * g->Ci;
  long M = g->B * g->OC * g->OR * g->OD;
  memset(dx, 0, sizeof(T) * g->B * g->IC * g->IR * g->ID * g->Ci);
  if (M == 0 || K == 0 || g->Co == 0) return 0;
  long mb = FN(block_rows_)(g);
  T *col = (T *)malloc(sizeof(T) * mb * K);
  if (!col) return -1;
  for (long m0 = 0; m0 < M; m0 += mb) {
    long rows = (M - m0 < mb) ? M - m0 : mb;
    FN(gemm_)(0, 1, rows, K, g->Co, dy + m0 * g->Co, g->Co, w, g->Co, (T)0, col, K);
    for (long i = 0; i < rows; ++i) FN(col2im_row_add_)(g, dx, m0 + i, col + i * K);
  }
  free(col);
  return 0;
}

/* dW = im2col(X)^T * dY.  Restates owl_ndarray_conv_impl.h:720-888 and
 * :1380-1440: the same column matrix reduced over output pixels, written in
 * the kernel's [kc][kr][kd][ci][co] order. */
static int FN(conv_bwd_kernel_)(const geom_t *g, const T *x, T *dw, const T *dy) {
  long K = g->KC * g->KR * g->KD * g->Ci;
  long M = g->B * g->OC * g->OR * g->OD;
  memset(dw, 0, sizeof(T) * K * g->Co);
  if (M == 0 || K == 0 || g->Co == 0) return 0;
  long mb = FN(block_rows_)(g);
  T *col = (T *)malloc(sizeof(T) * mb * K);
  if (!col) return -1;
  for (long m0 = 0; m0 < M; m0 += mb) {
    long rows = (M - m0 < mb) ? M - m0 : mb;
    for (long i = 0; i < rows; ++i) FN(im2col_row_)(g, x, m0 + i, col + i * K);
    FN(gemm_)(1, 0, K, g->Co, rows, col, K, dy + m0 * g->Co, g->Co, (T)1, dw, g->Co);
  }
  free(col);
  return 0;
}

/* ---- pooling: exact restatement (bit-exact results required) ---------- */

/* Window scan shared by every pooling function: columns outer, then rows,
 * then depths, skipping out-of-range taps (owl_ndarray_pool_impl.h:60-77,
 * :282-300). mode 0 = max, 1 = avg. */
static void FN(pool_fwd_)(const pgeom_t *g, const T *x, T *y, int64_t *argmax, int mode) {
  long chs = g->Ch;
  for (long i = 0; i < g->B; ++i) {
    const T *xb = x + i * g->IC * g->IR * g->ID * chs;
    long xbase = i * g->IC * g->IR * g->ID * chs;
    for (long j = 0; j < g->OC; ++j)
      for (long k = 0; k < g->OR; ++k)
        for (long d = 0; d < g->OD; ++d) {
          long cs = j * g->sc - g->pc, rs = k * g->sr - g->pr, ds = d * g->sd - g->pd;
          T *yo = y + (((i * g->OC + j) * g->OR + k) * g->OD + d) * chs;
          int64_t *ao = argmax ? argmax + (((i * g->OC + j) * g->OR + k) * g->OD + d) * chs : 0;
          for (long l = 0; l < chs; ++l) {
            T acc = mode == 0 ? (T)(-INFINITY) : (T)0;
            long midx = -1;
            int cnt = 0;
            for (long a = cs; a < cs + g->KC; ++a)
              for (long b = rs; b < rs + g->KR; ++b)
                for (long c = ds; c < ds + g->KD; ++c) {
                  if (a >= 0 && a < g->IC && b >= 0 && b < g->IR && c >= 0 && c < g->ID) {
                    long off = ((a * g->IR + b) * g->ID + c) * chs + l;
                    T t = xb[off];
                    if (mode == 0) {
                      if (LT(acc, t)) { acc = t; midx = xbase + off; }
                    } else {
                      acc += t;
                    }
                    cnt++;
                  }
                }
            if (mode == 0) yo[l] = acc;
            else yo[l] = acc / cnt; /* owl_ndarray_pool_stub.c:39-41: a / b */
            if (ao) ao[l] = (int64_t)midx;
          }
        }
  }
}

/* Backward: re-derive the window, route dY to the recomputed argmax
 * (max_idx starts at 0, owl_ndarray_pool_impl.h:167) or spread dY/count to
 * every in-range element (:189-191), accumulating with += in loop order. */
static void FN(pool_bwd_)(const pgeom_t *g, const T *x, const T *dy, T *dx, int mode) {
  long chs = g->Ch;
  memset(dx, 0, sizeof(T) * g->B * g->IC * g->IR * g->ID * chs);
  for (long i = 0; i < g->B; ++i) {
    long xbase = i * g->IC * g->IR * g->ID * chs;
    for (long j = 0; j < g->OC; ++j)
      for (long k = 0; k < g->OR; ++k)
        for (long d = 0; d < g->OD; ++d) {
          long cs = j * g->sc - g->pc, rs = k * g->sr - g->pr, ds = d * g->sd - g->pd;
          const T *go = dy + (((i * g->OC + j) * g->OR + k) * g->OD + d) * chs;
          for (long l = 0; l < chs; ++l) {
            T m = go[l];
            T acc = (T)(-INFINITY);
            long midx = 0;
            int cnt = 0;
            for (long a = cs; a < cs + g->KC; ++a)
              for (long b = rs; b < rs + g->KR; ++b)
                for (long c = ds; c < ds + g->KD; ++c)
                  if (a >= 0 && a < g->IC && b >= 0 && b < g->IR && c >= 0 && c < g->ID) {
                    long off = xbase + ((a * g->IR + b) * g->ID + c) * chs + l;
                    cnt++;
                    if (mode == 0) {
                      T t = x[off];
                      if (LT(acc, t)) { acc = t; midx = off; }
                    }
                  }
            if (mode == 0) {
              dx[midx] += m;
            } else {
              for (long a = cs; a < cs + g->KC; ++a)
                for (long b = rs; b < rs + g->KR; ++b)
                  for (long c = ds; c < ds + g->KD; ++c)
                    if (a >= 0 && a < g->IC && b >= 0 && b < g->IR && c >= 0 && c < g->ID) {
                      long off = xbase + ((a * g->IR + b) * g->ID + c) * chs + l;
                      dx[off] += m / cnt;
                    }
            }
          }
        }
  }
}

#undef FN
#undef CAT
#undef CAT_
