// api.cu -- the C ABI of libowlgpu (declared in include/owlgpu.h).
//
// Two families per Owl stub:
//   owl_<kind>_ndarray_<op>(host pointers, Owl stub arguments)
//       synchronous drop-in for the C stub of the same OCaml external name;
//       stages inputs to the GPU, runs, copies outputs back.
//   owlgpu_<kind>_ndarray_<op>(device pointers, Owl stub arguments,
//                              precision, stream)
//       asynchronous, device resident.
// Both turn the stub arguments into a ConvGeom / PoolGeom with the padding
// rules of the Owl stubs and call the compute layer.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/owlgpu.h"
#include "common.cuh"

namespace owlgpu {

std::atomic<uint64_t> g_launches{0};

static thread_local std::string t_error;

void set_error(const std::string &msg) { t_error = msg; }
const char *get_error() { return t_error.c_str(); }

int cuda_fail(cudaError_t e, const char *where) {
  set_error(std::string(where) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? kErrNoMem : kErrCuda;
}

int scratch_alloc(void **p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  if (bytes == 0) return kOk;
  cudaError_t e = cudaMallocAsync(p, bytes, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_fail(e, "cudaMallocAsync(scratch)");
  }
  return kOk;
}

void scratch_free(void *p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

static thread_local bool t_tc_launched = false;
void note_tc_launch() { t_tc_launched = true; }
bool take_tc_launched() {
  const bool v = t_tc_launched;
  t_tc_launched = false;
  return v;
}

// ---- dispatch between SIMT and tensor-core kernels -----------------------

static bool tc_requested(Dtype dt, int prec) { return dt == F32 && prec != OWLGPU_PREC_FP32; }

// Kernel family used by the calling thread's last convolution (reported by
// owlgpu_last_conv_path): 0 = CUDA-core (FP32/FP64), 1 = tcgen05 tensor cores.
static thread_local int t_last_path = -1;

// A float32 request for tensor-core precision runs on tcgen05 when the
// geometry is one the tensor-core kernels implement (strides up to 8, a halo
// that fits shared memory, no empty extents); otherwise it runs on the FP32
// CUDA-core kernels, which are at least as accurate.  The path taken is
// visible through owlgpu_last_conv_path().
int conv_fwd(Dtype dt, int prec, const ConvGeom &g, const void *x, const void *w, void *y,
             cudaStream_t s, const void *bias, int act) {
  if (tc_requested(dt, prec) && prec != OWLGPU_PREC_TF32) {
    // kernel = stride: a GEMM over the windows
    int rc = tc_conv_s2d(prec, false, g, (const float *)x, (const float *)w, (float *)y,
                         (const float *)bias, act, s);
    if (rc != kErrUnsupported) {
      t_last_path = 1;
      return rc;
    }
  }
  if (tc_requested(dt, prec)) {
    int rc = tc_conv_fwd(prec, g, (const float *)x, (const float *)w, (float *)y, s,
                         (const float *)bias, act);
    if (rc != kErrUnsupported) {
      t_last_path = 1;
      return rc;
    }
  }
  t_last_path = 0;
  int rc = simt_conv_fwd(dt, g, x, w, y, s);
  if (rc || (!bias && act == OWLGPU_ACT_NONE)) return rc;
  return bias_act_inplace(dt, y, bias, g.y_elems(), g.Co, act, s);
}

int conv_bwd_input(Dtype dt, int prec, const ConvGeom &g, void *dx, const void *w,
                   const void *dy, cudaStream_t s) {
  if (tc_requested(dt, prec)) {
    int rc = tc_conv_bwd_input(prec, g, (float *)dx, (const float *)w, (const float *)dy, s);
    if (rc != kErrUnsupported) {
      t_last_path = 1;
      return rc;
    }
  }
  t_last_path = 0;
  return simt_conv_bwd_input(dt, g, dx, w, dy, s);
}

int conv_bwd_kernel(Dtype dt, int prec, const ConvGeom &g, const void *x, void *dw,
                    const void *dy, cudaStream_t s) {
  if (tc_requested(dt, prec)) {
    // kernel = stride: a GEMM over the windows
    int rc = tc_conv_s2d(prec, true, g, (const float *)x, (const float *)dy, (float *)dw,
                         nullptr, 0, s);
    if (rc != kErrUnsupported) {
      t_last_path = 1;
      return rc;
    }
  }
  if (tc_requested(dt, prec)) {
    int rc = tc_conv_bwd_kernel(prec, g, (const float *)x, (float *)dw, (const float *)dy, s);
    if (rc != kErrUnsupported) {
      t_last_path = 1;
      return rc;
    }
  }
  t_last_path = 0;
  return simt_conv_bwd_kernel(dt, g, x, dw, dy, s);
}

// ---- argument checking and geometry construction -------------------------

static bool bad_dims(std::initializer_list<long> dims) {
  for (long d : dims)
    if (d < 0 || d > (1L << 30)) return true;
  return false;
}
static bool bad_pos(std::initializer_list<long> v) {
  for (long d : v)
    if (d < 1 || d > (1L << 20)) return true;
  return false;
}

static long keff(long k, long rate) { return k + (k - 1) * (rate - 1); }
static int fwd_pad(long padding, long stride, long out, long ke, long in) {
  if (padding == 1) return 0;
  long p = (stride * (out - 1) + ke - in) / 2;
  return (int)(p < 0 ? 0 : p);
}
static int bwd_pad(long stride, long out, long ke, long in) {
  long p = (stride * (out - 1) + ke - in) / 2;
  return (int)(p < 0 ? 0 : p);
}

static int invalid(const char *fn, const char *what) {
  set_error(std::string(fn) + ": " + what);
  return kErrInvalid;
}

// Build a ConvGeom.  `bwd` selects the backward padding rule; `rates` are
// (cols, rows, dpts) dilation rates, all 1 for the non-dilated stubs.
int make_conv(const char *fn, ConvGeom &g, long B, long IC, long IR, long ID, long Ci, long KC,
              long KR, long KD, long OC, long OR, long OD, long Co, long sc, long sr, long sd,
              long dc, long dr, long dd, bool bwd, long padding) {
  if (bad_dims({B, IC, IR, ID, Ci, KC, KR, KD, OC, OR, OD, Co}))
    return invalid(fn, "negative or oversized dimension");
  if (bad_pos({sc, sr, sd})) return invalid(fn, "stride must be >= 1");
  if (bad_pos({dc, dr, dd})) return invalid(fn, "dilation rate must be >= 1");
  if (!bwd && padding != 0 && padding != 1) return invalid(fn, "padding must be 0 (SAME) or 1 (VALID)");
  g.B = B; g.IC = IC; g.IR = IR; g.ID = ID; g.Ci = Ci;
  g.KC = KC; g.KR = KR; g.KD = KD;
  g.OC = OC; g.OR = OR; g.OD = OD; g.Co = Co;
  g.sc = (int)sc; g.sr = (int)sr; g.sd = (int)sd;
  g.dc = (int)dc; g.dr = (int)dr; g.dd = (int)dd;
  if (bwd) {
    g.pc = bwd_pad(sc, OC, keff(KC, dc), IC);
    g.pr = bwd_pad(sr, OR, keff(KR, dr), IR);
    g.pd = bwd_pad(sd, OD, keff(KD, dd), ID);
  } else {
    g.pc = fwd_pad(padding, sc, OC, keff(KC, dc), IC);
    g.pr = fwd_pad(padding, sr, OR, keff(KR, dr), IR);
    g.pd = fwd_pad(padding, sd, OD, keff(KD, dd), ID);
  }
  return kOk;
}

// The pooling padding flag: 0 = SAME, 1 = VALID, as for the convolutions (Owl's
// stubs read any value other than 1 as SAME; its OCaml layer passes only 0 or 1).
static int check_pool_padding(const char *fn, long padding) {
  if (padding != 0 && padding != 1) return invalid(fn, "padding must be 0 (SAME) or 1 (VALID)");
  return kOk;
}

static int make_pool(const char *fn, PoolGeom &g, long B, long IC, long IR, long ID, long Ch,
                     long KC, long KR, long KD, long OC, long OR, long OD, long sc, long sr,
                     long sd) {
  if (bad_dims({B, IC, IR, ID, Ch, KC, KR, KD, OC, OR, OD}))
    return invalid(fn, "negative or oversized dimension");
  if (bad_pos({sc, sr, sd})) return invalid(fn, "stride must be >= 1");
  g.B = B; g.IC = IC; g.IR = IR; g.ID = ID; g.Ch = Ch;
  g.KC = KC; g.KR = KR; g.KD = KD;
  g.OC = OC; g.OR = OR; g.OD = OD;
  g.sc = (int)sc; g.sr = (int)sr; g.sd = (int)sd;
  g.pc = g.pr = g.pd = 0;
  return kOk;
}

static int make_up(const char *fn, UpGeom &g, bool fwd, long B, long IC, long IR, long Ch,
                   long OC, long OR, long sc, long sr) {
  if (bad_dims({B, IC, IR, Ch, OC, OR})) return invalid(fn, "negative or oversized dimension");
  if (bad_pos({sc, sr})) return invalid(fn, "scale must be >= 1");
  // forward: the output is exactly the repeated input (Owl's repeat); the
  // backward stub accepts any output extent but needs an input position
  // to clamp into
  if (fwd && (OC != IC * sc || OR != IR * sr))
    return invalid(fn, "output must be input_cols * col_scale x input_rows * row_scale");
  if (!fwd && B * Ch > 0 && (IC == 0 || IR == 0) && OC * OR > 0)
    return invalid(fn, "empty input with a non-empty output gradient");
  g.B = B; g.IC = IC; g.IR = IR; g.Ch = Ch; g.OC = OC; g.OR = OR;
  g.sc = (int)sc; g.sr = (int)sr;
  return kOk;
}

// ---- host drop-in staging --------------------------------------------------

static std::atomic<int> g_precision{-1};
static std::atomic<long long> g_wait_limit{4000000000LL};

long long wait_limit() { return g_wait_limit.load(); }
long long set_wait_limit(long long cycles) {
  return g_wait_limit.exchange(cycles > 0 ? cycles : 4000000000LL);
}
static std::atomic<int> g_device{0};

static int default_precision() {
  int p = g_precision.load();
  if (p >= 0) return p;
  const char *e = getenv("OWLGPU_PRECISION");
  p = OWLGPU_PREC_FP32;
  if (e) {
    if (!strcmp(e, "tf32")) p = OWLGPU_PREC_TF32;
    else if (!strcmp(e, "bf16")) p = OWLGPU_PREC_BF16;
    else if (!strcmp(e, "bf16x3")) p = OWLGPU_PREC_BF16X3;
  }
  int expected = -1;
  g_precision.compare_exchange_strong(expected, p);
  return g_precision.load();
}

// Per host thread: a compute stream and two copy streams (host-to-device,
// device-to-host), plus events to order them, reused across calls.
struct HostStream {
  cudaStream_t s = nullptr, cin = nullptr, cout = nullptr;
  int device = -1;
  std::vector<cudaEvent_t> ev;
};
static thread_local HostStream t_stream;

static int host_stream(HostStream **out) {
  int dev = g_device.load();
  if (t_stream.s == nullptr || t_stream.device != dev) {
    OWL_CUDA(cudaSetDevice(dev));
    // Keep freed staging memory cached in the device's default pool so that
    // repeated drop-in calls do not return it to the driver at every sync.
    cudaMemPool_t pool;
    OWL_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t keep = UINT64_MAX;
    OWL_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    cudaStream_t st[3];
    for (auto &x : st) OWL_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
    t_stream.s = st[0];
    t_stream.cin = st[1];
    t_stream.cout = st[2];
    t_stream.ev.clear();
    t_stream.device = dev;
  } else {
    OWL_CUDA(cudaSetDevice(dev));
  }
  *out = &t_stream;
  return kOk;
}

static int host_events(HostStream &hs, size_t n) {
  while (hs.ev.size() < n) {
    cudaEvent_t e;
    OWL_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    hs.ev.push_back(e);
  }
  return kOk;
}

struct Buf {
  const void *host;  // source (inputs) or destination (outputs)
  size_t bytes;
  bool in, out;
  bool batched;      // leading axis is the batch: staged chunk by chunk
  void *dev = nullptr;
};

static bool page_locked(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Number of batch chunks for a staged call: about 24 MB of batched traffic
// per chunk, at most 8, at most one sample per chunk.  Copies from or to
// pageable host memory block the calling thread, which would serialise the
// pipeline, so a call with any pageable batched buffer is staged whole.
static int chunks_for(const std::vector<Buf> &bufs, int64_t batch) {
  size_t moved = 0;
  for (auto &b : bufs) {
    if (!b.batched || b.bytes == 0) continue;
    if (!page_locked(b.host)) return 1;
    moved += b.bytes;
  }
  int64_t c = (int64_t)(moved / (24u << 20));
  return (int)std::max<int64_t>(1, std::min<int64_t>({c, 8, batch}));
}

// Stage `bufs` to the device, run `body(dev pointers, b0, nb, stream)` over
// the batch in `chunks` pieces, copy the outputs back and wait.  With more
// than one chunk the host-to-device copy of chunk c+1, the compute of chunk
// c and the device-to-host copy of chunk c-1 run concurrently on three
// streams; only calls whose every batch sample is independent are chunked,
// and they give the same results as one call.  Device memory comes from the
// stream-ordered pool, so repeated calls of the same size reuse it.
// `finish(dev pointers, stream)` runs on the compute stream after the last
// chunk, before the unbatched outputs are copied back.
struct NoFinish {
  int operator()(std::vector<void *> &, cudaStream_t) const { return kOk; }
};
template <typename F, typename Fin = NoFinish>
static int host_call(std::vector<Buf> bufs, int64_t batch, int chunks, F body,
                     Fin finish = NoFinish()) {
  HostStream *hs;
  int rc = host_stream(&hs);
  if (rc) return rc;
  if (batch <= 0) chunks = 1;
  rc = host_events(*hs, 2 * (size_t)chunks);
  if (rc) return rc;
  take_tc_launched();  // clear: the status words are read below only if this call used them
  // one piece: copies and compute in order on one stream (no cross-stream
  // events, one synchronisation)
  const bool one = chunks == 1;
  cudaStream_t cin = one ? hs->s : hs->cin, cout = one ? hs->s : hs->cout;
  for (auto &b : bufs) {
    if (b.bytes == 0) continue;
    rc = scratch_alloc(&b.dev, b.bytes, cin);
    if (rc) break;
    if (b.in && !b.batched) {
      cudaError_t e = cudaMemcpyAsync(b.dev, b.host, b.bytes, cudaMemcpyHostToDevice, cin);
      if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpyAsync(H2D)"); break; }
    }
  }
  std::vector<void *> ptrs;
  for (auto &b : bufs) ptrs.push_back(b.dev);
  for (int c = 0; rc == kOk && c < chunks; ++c) {
    const int64_t b0 = batch * c / chunks, b1 = batch * (c + 1) / chunks;
    cudaEvent_t ein = hs->ev[2 * c], ecomp = hs->ev[2 * c + 1];
    for (auto &b : bufs) {
      if (!b.in || !b.batched || b.bytes == 0) continue;
      const size_t per = b.bytes / (size_t)batch;
      cudaError_t e = cudaMemcpyAsync((char *)b.dev + per * b0, (const char *)b.host + per * b0,
                                      per * (b1 - b0), cudaMemcpyHostToDevice, cin);
      if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpyAsync(H2D)"); break; }
    }
    if (rc) break;
    // errors leave the loop (not the function): the scratch buffers are
    // freed and the streams synchronised below on every path
    if (!one) {
      cudaError_t e = cudaEventRecord(ein, hs->cin);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(hs->s, ein, 0);
      if (e != cudaSuccess) { rc = cuda_fail(e, "cudaStreamWaitEvent(copy-in)"); break; }
    }
    rc = body(ptrs, b0, b1 - b0, hs->s);
    if (rc) break;
    if (!one) {
      cudaError_t e = cudaEventRecord(ecomp, hs->s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(hs->cout, ecomp, 0);
      if (e != cudaSuccess) { rc = cuda_fail(e, "cudaStreamWaitEvent(compute)"); break; }
    }
    for (auto &b : bufs) {
      if (!b.out || !b.batched || b.bytes == 0) continue;
      const size_t per = b.bytes / (size_t)batch;
      cudaError_t e = cudaMemcpyAsync((char *)b.host + per * b0, (char *)b.dev + per * b0,
                                      per * (b1 - b0), cudaMemcpyDeviceToHost, cout);
      if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpyAsync(D2H)"); break; }
    }
  }
  if (rc == kOk) rc = finish(ptrs, hs->s);
  if (rc == kOk) {
    for (auto &b : bufs) {
      if (!b.out || b.batched || b.bytes == 0) continue;
      cudaError_t e = cudaMemcpyAsync(const_cast<void *>(b.host), b.dev, b.bytes,
                                      cudaMemcpyDeviceToHost, hs->s);
      if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpyAsync(D2H)"); break; }
    }
  }
  // the watchdog status words ride on the compute stream's synchronisation
  const bool tc = take_tc_launched();
  if (rc == kOk && tc) rc = tc_status_enqueue(hs->s);
  cudaError_t e1 = one ? cudaSuccess : cudaStreamSynchronize(hs->cin);
  cudaError_t e2 = cudaStreamSynchronize(hs->s);
  cudaError_t e3 = one ? cudaSuccess : cudaStreamSynchronize(hs->cout);
  for (auto &b : bufs) scratch_free(b.dev, hs->s);
  cudaError_t e = e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3;
  if (rc == kOk && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
  if (rc == kOk && tc) {
    int st = 0;
    rc = tc_status_take(&st, hs->s);
    if (rc == kOk && st) {
      set_error("a tensor-core kernel gave up waiting on one of its pipeline barriers");
      rc = kErrTimeout;
    }
  }
  return rc;
}

// Element kind of each C-ABI element type.
template <typename T>
struct ElemKind;
template <>
struct ElemKind<float> { static constexpr Dtype v = F32; };
template <>
struct ElemKind<double> { static constexpr Dtype v = F64; };
template <>
struct ElemKind<owlgpu_complex32> { static constexpr Dtype v = C32; };
template <>
struct ElemKind<owlgpu_complex64> { static constexpr Dtype v = C64; };
static_assert(sizeof(owlgpu_complex32) == sizeof(c32) && sizeof(owlgpu_complex64) == sizeof(c64),
              "complex layouts");

template <typename T>
static Dtype dtype_of() { return ElemKind<T>::v; }

// Conv op kinds.
enum ConvOp { OP_FWD, OP_BWDI, OP_BWDK };

template <typename T>
static int conv_device(ConvOp op, const ConvGeom &g, void *a, void *b, void *c, int prec,
                       cudaStream_t s) {
  Dtype dt = dtype_of<T>();
  if (op == OP_FWD) return conv_fwd(dt, prec, g, a, b, c, s);
  if (op == OP_BWDI) return conv_bwd_input(dt, prec, g, a, b, c, s);
  return conv_bwd_kernel(dt, prec, g, a, b, c, s);
}

// Host drop-in for a conv stub: argument roles follow the Owl stubs.
//   FWD : (X in, W in, Y out)
//   BWDI: (dX out, W in, dY in)
//   BWDK: (X in, dW out, dY in)
template <typename T>
static int conv_host(ConvOp op, const ConvGeom &g, const void *a, const void *b, const void *c) {
  size_t xb = sizeof(T) * g.x_elems(), wb = sizeof(T) * g.w_elems(), yb = sizeof(T) * g.y_elems();
  // forward and backward_input are independent per batch sample: staged in
  // chunks.  A float32 backward_kernel is staged in chunks too: each chunk's
  // weight gradient lands in its own partial, and the partials are summed
  // in chunk order at the end (deterministic), so the kernels run while the
  // later chunks are still being copied in.
  const bool bwdk = op == OP_BWDK;
  const bool chunk = !bwdk || dtype_of<T>() == F32;
  std::vector<Buf> bufs;
  if (op == OP_FWD)
    bufs = {{a, xb, true, false, chunk}, {b, wb, true, false, false}, {c, yb, false, true, chunk}};
  else if (op == OP_BWDI)
    bufs = {{a, xb, false, true, chunk}, {b, wb, true, false, false}, {c, yb, true, false, chunk}};
  else
    bufs = {{a, xb, true, false, chunk}, {b, wb, false, true, false}, {c, yb, true, false, chunk}};
  int prec = default_precision();
  const int chunks = chunk ? chunks_for(bufs, g.B) : 1;
  const int64_t xs = g.x_elems() / std::max<int64_t>(g.B, 1);
  const int64_t ys = g.y_elems() / std::max<int64_t>(g.B, 1);
  const long long welems = g.w_elems();
  float *part = nullptr;  // [chunks][welems] when a backward_kernel is split
  int ci = 0;
  const bool split = bwdk && chunks > 1;
  int rc = host_call(
      bufs, g.B, chunks,
      [&](std::vector<void *> &p, int64_t b0, int64_t nb, cudaStream_t s) {
        ConvGeom gc = g;
        gc.B = nb;
        T *x = (T *)p[0] + (chunk ? b0 * xs : 0);
        T *y = (T *)p[2] + (chunk ? b0 * ys : 0);
        void *w = p[1];
        if (split) {
          if (ci == 0) {
            const int r = scratch_alloc((void **)&part, sizeof(float) * (size_t)welems * chunks, s);
            if (r) return r;
          }
          w = part + (size_t)welems * ci++;
        }
        return conv_device<T>(op, gc, x, w, y, prec, s);
      },
      [&](std::vector<void *> &p, cudaStream_t s) {
        if (!split) return (int)kOk;
        return sum_partials_f32(part, (float *)p[1], welems, chunks, s);
      });
  if (part) {
    // the call has synchronised its streams; the pool takes the memory back
    HostStream *hs;
    if (host_stream(&hs) == kOk) scratch_free(part, hs->s);
  }
  return rc;
}

template <typename T>
static int pool_fwd_host(PoolMode mode, const PoolGeom &g, const void *x, void *y,
                         int64_t *arg) {
  // argmax holds flat indices into the whole input: staged in one piece.
  const bool chunk = arg == nullptr;
  std::vector<Buf> bufs = {{x, sizeof(T) * g.x_elems(), true, false, chunk},
                           {y, sizeof(T) * g.y_elems(), false, true, chunk}};
  if (arg) bufs.push_back({arg, sizeof(int64_t) * g.y_elems(), false, true, false});
  const int chunks = chunk ? chunks_for(bufs, g.B) : 1;
  const int64_t xs = g.x_elems() / std::max<int64_t>(g.B, 1);
  const int64_t ys = g.y_elems() / std::max<int64_t>(g.B, 1);
  return host_call(bufs, g.B, chunks,
                   [&](std::vector<void *> &p, int64_t b0, int64_t nb, cudaStream_t s) {
    PoolGeom gc = g;
    gc.B = nb;
    return pool_fwd(dtype_of<T>(), mode, gc, (T *)p[0] + b0 * xs, (T *)p[1] + b0 * ys,
                    arg ? (int64_t *)p[2] : nullptr, s);
  });
}

// Upsampling is independent per sample: staged in batch chunks.  `x` is the
// array read (input, or dy), `y` the array written (output, or dx).
template <typename T>
static int up_host(bool fwd, const UpGeom &g, const void *x, void *y) {
  const size_t xb = sizeof(T) * (size_t)(fwd ? g.x_elems() : g.y_elems());
  const size_t yb = sizeof(T) * (size_t)(fwd ? g.y_elems() : g.x_elems());
  std::vector<Buf> bufs = {{x, xb, true, false, true}, {y, yb, false, true, true}};
  const int chunks = chunks_for(bufs, g.B);
  const int64_t xs = (int64_t)(xb / sizeof(T)) / std::max<int64_t>(g.B, 1);
  const int64_t ys = (int64_t)(yb / sizeof(T)) / std::max<int64_t>(g.B, 1);
  return host_call(bufs, g.B, chunks,
                   [&](std::vector<void *> &p, int64_t b0, int64_t nb, cudaStream_t s) {
    UpGeom gc = g;
    gc.B = nb;
    const T *px = (const T *)p[0] + b0 * xs;
    T *py = (T *)p[1] + b0 * ys;
    return fwd ? upsample_fwd(dtype_of<T>(), gc, px, py, s)
               : upsample_bwd(dtype_of<T>(), gc, py, px, s);
  });
}

template <typename T>
static int pool_bwd_host(PoolMode mode, const PoolGeom &g, const void *x, const void *dy,
                         void *dx) {
  // Average pooling never reads X (Owl passes a dummy there) and is
  // independent per sample; max pooling routes degenerate windows to flat
  // element 0 of the whole input, so it is staged in one piece.
  const bool chunk = mode == POOL_AVG;
  std::vector<Buf> bufs = {
      {x, mode == POOL_MAX ? sizeof(T) * g.x_elems() : 0, true, false, false},
      {dy, sizeof(T) * g.y_elems(), true, false, chunk},
      {dx, sizeof(T) * g.x_elems(), false, true, chunk}};
  const int chunks = chunk ? chunks_for(bufs, g.B) : 1;
  const int64_t xs = g.x_elems() / std::max<int64_t>(g.B, 1);
  const int64_t ys = g.y_elems() / std::max<int64_t>(g.B, 1);
  return host_call(bufs, g.B, chunks,
                   [&](std::vector<void *> &p, int64_t b0, int64_t nb, cudaStream_t s) {
    PoolGeom gc = g;
    gc.B = nb;
    const T *px = chunk ? nullptr : (const T *)p[0];
    return pool_bwd(dtype_of<T>(), mode, gc, px, (T *)p[1] + b0 * ys, (T *)p[2] + b0 * xs, s);
  });
}

}  // namespace owlgpu

using namespace owlgpu;

// ===========================================================================
// Exported C ABI
// ===========================================================================

extern "C" {

const char *owlgpu_last_error(void) { return get_error(); }
const char *owlgpu_version(void) { return "owlgpu 0.1 (sm_103a)"; }

int owlgpu_set_precision(int p) {
  if (p < OWLGPU_PREC_FP32 || p > OWLGPU_PREC_BF16X3) {
    set_error("owlgpu_set_precision: unknown precision");
    return kErrInvalid;
  }
  int prev = default_precision();
  g_precision.store(p);
  return prev;
}
int owlgpu_get_precision(void) { return default_precision(); }
long long owlgpu_set_wait_limit(long long cycles) { return set_wait_limit(cycles); }
uint64_t owlgpu_launch_count(void) { return g_launches.load(); }
int owlgpu_last_conv_path(void) { return t_last_path; }
int owlgpu_device_status(void) {
  HostStream *hs;
  int rc = host_stream(&hs);
  if (rc) return rc;
  int v = 0;
  rc = tc_read_status(&v, hs->s);
  if (rc) return rc;
  if (v) {
    set_error("a tensor-core kernel gave up waiting on one of its pipeline barriers");
    return kErrTimeout;
  }
  return kOk;
}
int owlgpu_set_device(int d) {
  int n = 0;
  OWL_CUDA(cudaGetDeviceCount(&n));
  if (d < 0 || d >= n) { set_error("owlgpu_set_device: no such device"); return kErrInvalid; }
  g_device.store(d);
  return kOk;
}
int owlgpu_trim(void) {
  int dev = g_device.load();
  cudaMemPool_t pool;
  OWL_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  OWL_CUDA(cudaDeviceSynchronize());
  OWL_CUDA(cudaMemPoolTrimTo(pool, 0));
  return weights_drop_all();
}
int owlgpu_weights_declare(const void *kernel, uint64_t version) {
  if (!kernel) {
    set_error("owlgpu_weights_declare: null kernel pointer");
    return kErrInvalid;
  }
  return weights_declare(kernel, version);
}
int owlgpu_weights_forget(const void *kernel) { return weights_forget(kernel); }

// ---- device buffers and streams for callers without the CUDA runtime --------

int owlgpu_stream_create(void **stream) {
  if (!stream) {
    set_error("owlgpu_stream_create: null result pointer");
    return kErrInvalid;
  }
  cudaStream_t s = nullptr;
  OWL_CUDA(cudaSetDevice(g_device.load()));
  OWL_CUDA(cudaStreamCreate(&s));
  *stream = (void *)s;
  return kOk;
}
int owlgpu_stream_destroy(void *stream) {
  if (stream) OWL_CUDA(cudaStreamDestroy((cudaStream_t)stream));
  return kOk;
}
int owlgpu_stream_synchronize(void *stream) {
  OWL_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return kOk;
}
int owlgpu_device_alloc(void **ptr, uint64_t bytes, void *stream) {
  if (!ptr) {
    set_error("owlgpu_device_alloc: null result pointer");
    return kErrInvalid;
  }
  *ptr = nullptr;
  OWL_CUDA(cudaSetDevice(g_device.load()));
  return scratch_alloc(ptr, (size_t)bytes, (cudaStream_t)stream);
}
int owlgpu_device_free(void *ptr, void *stream) {
  if (ptr) OWL_CUDA(cudaFreeAsync(ptr, (cudaStream_t)stream));
  return kOk;
}
int owlgpu_copy_to_device(void *dst, const void *src, uint64_t bytes, void *stream) {
  if (bytes == 0) return kOk;
  OWL_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  OWL_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return kOk;
}
int owlgpu_copy_to_host(void *dst, const void *src, uint64_t bytes, void *stream) {
  if (bytes == 0) return kOk;
  OWL_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  OWL_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return kOk;
}

// ---- 2-D conv (GEBP spatial family and its im2col / dilated spellings) ----

#define CONV2D_FWD(KIND, T, NAME, DIL)                                                        \
  int owl_##KIND##_ndarray_##NAME(const T *input, const T *kernel, T *output, long batches,  \
                                  long input_cols, long input_rows, long in_channel,          \
                                  long kernel_cols, long kernel_rows, long output_cols,       \
                                  long output_rows, long out_channel, long row_stride,        \
                                  long col_stride, long padding, long row_in_stride,          \
                                  long col_in_stride) {                                       \
    ConvGeom g;                                                                               \
    int rc = make_conv(#NAME, g, batches, input_cols, input_rows, 1, in_channel, kernel_cols, \
                       kernel_rows, 1, output_cols, output_rows, 1, out_channel, col_stride,  \
                       row_stride, 1, DIL ? col_in_stride : 1, DIL ? row_in_stride : 1, 1,    \
                       false, padding);                                                       \
    if (rc) return rc;                                                                        \
    return conv_host<T>(OP_FWD, g, input, kernel, output);                                    \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_##NAME(const T *input, const T *kernel, T *output,            \
                                     long batches, long input_cols, long input_rows,          \
                                     long in_channel, long kernel_cols, long kernel_rows,     \
                                     long output_cols, long output_rows, long out_channel,    \
                                     long row_stride, long col_stride, long padding,          \
                                     long row_in_stride, long col_in_stride, int precision,   \
                                     void *stream) {                                          \
    ConvGeom g;                                                                               \
    int rc = make_conv(#NAME, g, batches, input_cols, input_rows, 1, in_channel, kernel_cols, \
                       kernel_rows, 1, output_cols, output_rows, 1, out_channel, col_stride,  \
                       row_stride, 1, DIL ? col_in_stride : 1, DIL ? row_in_stride : 1, 1,    \
                       false, padding);                                                       \
    if (rc) return rc;                                                                        \
    return conv_device<T>(OP_FWD, g, (void *)input, (void *)kernel, output, precision,        \
                          (cudaStream_t)stream);                                              \
  }

#define CONV2D_BWD(KIND, T, NAME, OP, DIL, A_T, B_T, C_T, A_N, B_N, C_N)                       \
  int owl_##KIND##_ndarray_##NAME(A_T A_N, B_T B_N, C_T C_N, long batches, long input_cols,   \
                                  long input_rows, long in_channel, long kernel_cols,         \
                                  long kernel_rows, long output_cols, long output_rows,       \
                                  long out_channel, long row_stride, long col_stride,         \
                                  long row_in_stride, long col_in_stride) {                   \
    ConvGeom g;                                                                               \
    int rc = make_conv(#NAME, g, batches, input_cols, input_rows, 1, in_channel, kernel_cols, \
                       kernel_rows, 1, output_cols, output_rows, 1, out_channel, col_stride,  \
                       row_stride, 1, DIL ? col_in_stride : 1, DIL ? row_in_stride : 1, 1,    \
                       true, 0);                                                              \
    if (rc) return rc;                                                                        \
    return conv_host<T>(OP, g, A_N, B_N, C_N);                                                \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_##NAME(A_T A_N, B_T B_N, C_T C_N, long batches,               \
                                     long input_cols, long input_rows, long in_channel,       \
                                     long kernel_cols, long kernel_rows, long output_cols,    \
                                     long output_rows, long out_channel, long row_stride,     \
                                     long col_stride, long row_in_stride, long col_in_stride, \
                                     int precision, void *stream) {                           \
    ConvGeom g;                                                                               \
    int rc = make_conv(#NAME, g, batches, input_cols, input_rows, 1, in_channel, kernel_cols, \
                       kernel_rows, 1, output_cols, output_rows, 1, out_channel, col_stride,  \
                       row_stride, 1, DIL ? col_in_stride : 1, DIL ? row_in_stride : 1, 1,    \
                       true, 0);                                                              \
    if (rc) return rc;                                                                        \
    return conv_device<T>(OP, g, (void *)A_N, (void *)B_N, (void *)C_N, precision,            \
                          (cudaStream_t)stream);                                              \
  }

#define CONV2D_ALL(KIND, T)                                                                    \
  CONV2D_FWD(KIND, T, conv_spatial, 0)                                                        \
  CONV2D_FWD(KIND, T, conv_spatial_im2col, 0)                                                 \
  CONV2D_FWD(KIND, T, conv_dilated_spatial_im2col, 1)                                         \
  CONV2D_BWD(KIND, T, conv_spatial_backward_input, OP_BWDI, 0, T *, const T *, const T *,     \
             input_grad, kernel, output_grad)                                                 \
  CONV2D_BWD(KIND, T, conv_spatial_backward_input_im2col, OP_BWDI, 0, T *, const T *,         \
             const T *, input_grad, kernel, output_grad)                                      \
  CONV2D_BWD(KIND, T, conv_dilated_spatial_backward_input_im2col, OP_BWDI, 1, T *, const T *, \
             const T *, input_grad, kernel, output_grad)                                      \
  CONV2D_BWD(KIND, T, conv_spatial_backward_kernel, OP_BWDK, 0, const T *, T *, const T *,    \
             input, kernel_grad, output_grad)                                                 \
  CONV2D_BWD(KIND, T, conv_spatial_backward_kernel_im2col, OP_BWDK, 0, const T *, T *,        \
             const T *, input, kernel_grad, output_grad)                                      \
  CONV2D_BWD(KIND, T, conv_dilated_spatial_backward_kernel_im2col, OP_BWDK, 1, const T *,     \
             T *, const T *, input, kernel_grad, output_grad)

CONV2D_ALL(float32, float)
CONV2D_ALL(float64, double)
CONV2D_ALL(complex32, owlgpu_complex32)
CONV2D_ALL(complex64, owlgpu_complex64)

// ---- 3-D conv (cuboid im2col family and dilated cuboid) ---------------------

#define CONV3D_FWD(KIND, T)                                                                    \
  int owl_##KIND##_ndarray_conv_cuboid_im2col(                                                \
      const T *input, const T *kernel, T *output, long batches, long input_cols,              \
      long input_rows, long input_dpts, long in_channel, long kernel_cols, long kernel_rows,   \
      long kernel_dpts, long output_cols, long output_rows, long output_dpts,                  \
      long out_channel, long dpt_stride, long row_stride, long col_stride, long padding) {     \
    ConvGeom g;                                                                               \
    int rc = make_conv("conv_cuboid_im2col", g, batches, input_cols, input_rows, input_dpts,  \
                       in_channel, kernel_cols, kernel_rows, kernel_dpts, output_cols,        \
                       output_rows, output_dpts, out_channel, col_stride, row_stride,         \
                       dpt_stride, 1, 1, 1, false, padding);                                  \
    if (rc) return rc;                                                                        \
    return conv_host<T>(OP_FWD, g, input, kernel, output);                                    \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_conv_cuboid_im2col(                                             \
      const T *input, const T *kernel, T *output, long batches, long input_cols,              \
      long input_rows, long input_dpts, long in_channel, long kernel_cols, long kernel_rows,   \
      long kernel_dpts, long output_cols, long output_rows, long output_dpts,                  \
      long out_channel, long dpt_stride, long row_stride, long col_stride, long padding,       \
      int precision, void *stream) {                                                          \
    ConvGeom g;                                                                               \
    int rc = make_conv("conv_cuboid_im2col", g, batches, input_cols, input_rows, input_dpts,  \
                       in_channel, kernel_cols, kernel_rows, kernel_dpts, output_cols,        \
                       output_rows, output_dpts, out_channel, col_stride, row_stride,         \
                       dpt_stride, 1, 1, 1, false, padding);                                  \
    if (rc) return rc;                                                                        \
    return conv_device<T>(OP_FWD, g, (void *)input, (void *)kernel, output, precision,        \
                          (cudaStream_t)stream);                                              \
  }                                                                                           \
  int owl_##KIND##_ndarray_conv_dilated_cuboid_im2col(                                        \
      const T *input, const T *kernel, T *output, long batches, long input_cols,              \
      long input_rows, long input_dpts, long in_channel, long kernel_cols, long kernel_rows,   \
      long kernel_dpts, long output_cols, long output_rows, long output_dpts,                  \
      long out_channel, long dpt_stride, long row_stride, long col_stride,                     \
      long dpt_in_stride, long row_in_stride, long col_in_stride, long padding) {              \
    ConvGeom g;                                                                               \
    int rc = make_conv("conv_dilated_cuboid_im2col", g, batches, input_cols, input_rows,      \
                       input_dpts, in_channel, kernel_cols, kernel_rows, kernel_dpts,         \
                       output_cols, output_rows, output_dpts, out_channel, col_stride,        \
                       row_stride, dpt_stride, col_in_stride, row_in_stride, dpt_in_stride,   \
                       false, padding);                                                       \
    if (rc) return rc;                                                                        \
    return conv_host<T>(OP_FWD, g, input, kernel, output);                                    \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_conv_dilated_cuboid_im2col(                                     \
      const T *input, const T *kernel, T *output, long batches, long input_cols,              \
      long input_rows, long input_dpts, long in_channel, long kernel_cols, long kernel_rows,   \
      long kernel_dpts, long output_cols, long output_rows, long output_dpts,                  \
      long out_channel, long dpt_stride, long row_stride, long col_stride,                     \
      long dpt_in_stride, long row_in_stride, long col_in_stride, long padding,                \
      int precision, void *stream) {                                                          \
    ConvGeom g;                                                                               \
    int rc = make_conv("conv_dilated_cuboid_im2col", g, batches, input_cols, input_rows,      \
                       input_dpts, in_channel, kernel_cols, kernel_rows, kernel_dpts,         \
                       output_cols, output_rows, output_dpts, out_channel, col_stride,        \
                       row_stride, dpt_stride, col_in_stride, row_in_stride, dpt_in_stride,   \
                       false, padding);                                                       \
    if (rc) return rc;                                                                        \
    return conv_device<T>(OP_FWD, g, (void *)input, (void *)kernel, output, precision,        \
                          (cudaStream_t)stream);                                              \
  }

#define CONV3D_BWD(KIND, T, NAME, OP, DIL, A_T, B_T, C_T, A_N, B_N, C_N, DILARGS, DILVALS)      \
  int owl_##KIND##_ndarray_##NAME(A_T A_N, B_T B_N, C_T C_N, long batches, long input_cols,   \
                                  long input_rows, long input_dpts, long in_channel,          \
                                  long kernel_cols, long kernel_rows, long kernel_dpts,       \
                                  long output_cols, long output_rows, long output_dpts,       \
                                  long out_channel, long dpt_stride, long row_stride,         \
                                  long col_stride DILARGS) {                                  \
    ConvGeom g;                                                                               \
    int rc = make_conv(#NAME, g, batches, input_cols, input_rows, input_dpts, in_channel,     \
                       kernel_cols, kernel_rows, kernel_dpts, output_cols, output_rows,       \
                       output_dpts, out_channel, col_stride, row_stride, dpt_stride, DILVALS, \
                       true, 0);                                                              \
    if (rc) return rc;                                                                        \
    return conv_host<T>(OP, g, A_N, B_N, C_N);                                                \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_##NAME(A_T A_N, B_T B_N, C_T C_N, long batches,               \
                                     long input_cols, long input_rows, long input_dpts,       \
                                     long in_channel, long kernel_cols, long kernel_rows,     \
                                     long kernel_dpts, long output_cols, long output_rows,    \
                                     long output_dpts, long out_channel, long dpt_stride,     \
                                     long row_stride, long col_stride DILARGS, int precision, \
                                     void *stream) {                                          \
    ConvGeom g;                                                                               \
    int rc = make_conv(#NAME, g, batches, input_cols, input_rows, input_dpts, in_channel,     \
                       kernel_cols, kernel_rows, kernel_dpts, output_cols, output_rows,       \
                       output_dpts, out_channel, col_stride, row_stride, dpt_stride, DILVALS, \
                       true, 0);                                                              \
    if (rc) return rc;                                                                        \
    return conv_device<T>(OP, g, (void *)A_N, (void *)B_N, (void *)C_N, precision,            \
                          (cudaStream_t)stream);                                              \
  }

#define NODIL_ARGS
#define NODIL_VALS 1, 1, 1
#define DIL_ARGS , long dpt_in_stride, long row_in_stride, long col_in_stride
#define DIL_VALS col_in_stride, row_in_stride, dpt_in_stride

#define CONV3D_ALL(KIND, T)                                                                     \
  CONV3D_FWD(KIND, T)                                                                          \
  CONV3D_BWD(KIND, T, conv_cuboid_backward_input_im2col, OP_BWDI, 0, T *, const T *,           \
             const T *, input_grad, kernel, output_grad, NODIL_ARGS, NODIL_VALS)               \
  CONV3D_BWD(KIND, T, conv_cuboid_backward_kernel_im2col, OP_BWDK, 0, const T *, T *,          \
             const T *, input, kernel_grad, output_grad, NODIL_ARGS, NODIL_VALS)               \
  CONV3D_BWD(KIND, T, conv_dilated_cuboid_backward_input_im2col, OP_BWDI, 1, T *, const T *,   \
             const T *, input_grad, kernel, output_grad, DIL_ARGS, DIL_VALS)                   \
  CONV3D_BWD(KIND, T, conv_dilated_cuboid_backward_kernel_im2col, OP_BWDK, 1, const T *, T *,  \
             const T *, input, kernel_grad, output_grad, DIL_ARGS, DIL_VALS)

CONV3D_ALL(float32, float)
CONV3D_ALL(float64, double)
CONV3D_ALL(complex32, owlgpu_complex32)
CONV3D_ALL(complex64, owlgpu_complex64)

// ---- MEC and naive spellings of the conv stubs -------------------------------
// Owl's memory-efficient (MEC) and naive CPU algorithms compute the same
// functions as its GEBP / im2col ones, with the same stub arguments
// (owl_ndarray_conv_impl.h:1570-3086; Owl's unit_conv_mec_naive.ml runs its
// conv2d and conv3d test suites on them).  Host drop-in aliases of the same
// GPU implementation.

#define SP2_LONGS                                                                              \
  long batches, long input_cols, long input_rows, long in_channel, long kernel_cols,           \
      long kernel_rows, long output_cols, long output_rows, long out_channel, long row_stride, \
      long col_stride
#define SP2_VALS                                                                               \
  batches, input_cols, input_rows, in_channel, kernel_cols, kernel_rows, output_cols,          \
      output_rows, out_channel, row_stride, col_stride
#define CU3_LONGS                                                                              \
  long batches, long input_cols, long input_rows, long input_dpts, long in_channel,            \
      long kernel_cols, long kernel_rows, long kernel_dpts, long output_cols, long output_rows, \
      long output_dpts, long out_channel, long dpt_stride, long row_stride, long col_stride
#define CU3_VALS                                                                               \
  batches, input_cols, input_rows, input_dpts, in_channel, kernel_cols, kernel_rows,           \
      kernel_dpts, output_cols, output_rows, output_dpts, out_channel, dpt_stride, row_stride, \
      col_stride

#define CONV_SPELLINGS(KIND, T, SFX)                                                           \
  int owl_##KIND##_ndarray_conv_spatial_##SFX(const T *input, const T *kernel, T *output,     \
                                              SP2_LONGS, long padding, long row_in_stride,    \
                                              long col_in_stride) {                           \
    return owl_##KIND##_ndarray_conv_spatial(input, kernel, output, SP2_VALS, padding,        \
                                             row_in_stride, col_in_stride);                   \
  }                                                                                           \
  int owl_##KIND##_ndarray_conv_spatial_backward_input_##SFX(                                 \
      T *input_grad, const T *kernel, const T *output_grad, SP2_LONGS, long row_in_stride,    \
      long col_in_stride) {                                                                   \
    return owl_##KIND##_ndarray_conv_spatial_backward_input(input_grad, kernel, output_grad,  \
                                                            SP2_VALS, row_in_stride,          \
                                                            col_in_stride);                   \
  }                                                                                           \
  int owl_##KIND##_ndarray_conv_spatial_backward_kernel_##SFX(                                \
      const T *input, T *kernel_grad, const T *output_grad, SP2_LONGS, long row_in_stride,    \
      long col_in_stride) {                                                                   \
    return owl_##KIND##_ndarray_conv_spatial_backward_kernel(input, kernel_grad, output_grad, \
                                                             SP2_VALS, row_in_stride,         \
                                                             col_in_stride);                  \
  }                                                                                           \
  int owl_##KIND##_ndarray_conv_cuboid_##SFX(const T *input, const T *kernel, T *output,      \
                                             CU3_LONGS, long padding) {                       \
    return owl_##KIND##_ndarray_conv_cuboid_im2col(input, kernel, output, CU3_VALS, padding); \
  }                                                                                           \
  int owl_##KIND##_ndarray_conv_cuboid_backward_input_##SFX(                                  \
      T *input_grad, const T *kernel, const T *output_grad, CU3_LONGS) {                      \
    return owl_##KIND##_ndarray_conv_cuboid_backward_input_im2col(input_grad, kernel,         \
                                                                  output_grad, CU3_VALS);     \
  }                                                                                           \
  int owl_##KIND##_ndarray_conv_cuboid_backward_kernel_##SFX(                                 \
      const T *input, T *kernel_grad, const T *output_grad, CU3_LONGS) {                      \
    return owl_##KIND##_ndarray_conv_cuboid_backward_kernel_im2col(input, kernel_grad,        \
                                                                   output_grad, CU3_VALS);    \
  }

#define CONV_SPELLINGS_ALL(KIND, T) \
  CONV_SPELLINGS(KIND, T, mec)      \
  CONV_SPELLINGS(KIND, T, naive)

CONV_SPELLINGS_ALL(float32, float)
CONV_SPELLINGS_ALL(float64, double)
CONV_SPELLINGS_ALL(complex32, owlgpu_complex32)
CONV_SPELLINGS_ALL(complex64, owlgpu_complex64)

// ---- pooling -----------------------------------------------------------------

#define POOL2D_FWD(KIND, T, WHICH, MODE)                                                        \
  int owl_##KIND##_ndarray_##WHICH##_spatial(                                                  \
      const T *input, T *output, long batches, long input_cols, long input_rows,              \
      long in_channel, long kernel_cols, long kernel_rows, long output_cols, long output_rows, \
      long row_stride, long col_stride, long padding, long row_in_stride,                      \
      long col_in_stride) {                                                                    \
    (void)row_in_stride; (void)col_in_stride;                                                  \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_spatial", g, batches, input_cols, input_rows, 1, in_channel,  \
                       kernel_cols, kernel_rows, 1, output_cols, output_rows, 1, col_stride,  \
                       row_stride, 1);                                                        \
    if (rc) return rc;                                                                        \
    if (check_pool_padding(#WHICH, padding)) return kErrInvalid;                              \
    g.pr = fwd_pad(padding, row_stride, output_rows, kernel_rows, input_rows);                \
    g.pc = fwd_pad(padding, col_stride, output_cols, kernel_cols, input_cols);                \
    return pool_fwd_host<T>(MODE, g, input, output, nullptr);                                 \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_##WHICH##_spatial(                                               \
      const T *input, T *output, long batches, long input_cols, long input_rows,              \
      long in_channel, long kernel_cols, long kernel_rows, long output_cols, long output_rows, \
      long row_stride, long col_stride, long padding, long row_in_stride, long col_in_stride, \
      int precision, void *stream) {                                                          \
    (void)row_in_stride; (void)col_in_stride; (void)precision;                                 \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_spatial", g, batches, input_cols, input_rows, 1, in_channel,  \
                       kernel_cols, kernel_rows, 1, output_cols, output_rows, 1, col_stride,  \
                       row_stride, 1);                                                        \
    if (rc) return rc;                                                                        \
    if (check_pool_padding(#WHICH, padding)) return kErrInvalid;                              \
    g.pr = fwd_pad(padding, row_stride, output_rows, kernel_rows, input_rows);                \
    g.pc = fwd_pad(padding, col_stride, output_cols, kernel_cols, input_cols);                \
    return pool_fwd(dtype_of<T>(), MODE, g, input, output, nullptr, (cudaStream_t)stream);    \
  }

#define POOL2D_BWD(KIND, T, WHICH, MODE)                                                        \
  int owl_##KIND##_ndarray_##WHICH##_spatial_backward(                                         \
      const T *input, const T *output_grad, T *input_grad, long batches, long input_cols,     \
      long input_rows, long in_channel, long kernel_cols, long kernel_rows, long output_cols, \
      long output_rows, long row_stride, long col_stride, long pad_rows, long pad_cols) {      \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_spatial_backward", g, batches, input_cols, input_rows, 1,     \
                       in_channel, kernel_cols, kernel_rows, 1, output_cols, output_rows, 1,  \
                       col_stride, row_stride, 1);                                            \
    if (rc) return rc;                                                                        \
    g.pr = pad_rows < 0 ? 0 : (int)pad_rows;                                                  \
    g.pc = pad_cols < 0 ? 0 : (int)pad_cols;                                                  \
    return pool_bwd_host<T>(MODE, g, input, output_grad, input_grad);                         \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_##WHICH##_spatial_backward(                                      \
      const T *input, const T *output_grad, T *input_grad, long batches, long input_cols,     \
      long input_rows, long in_channel, long kernel_cols, long kernel_rows, long output_cols, \
      long output_rows, long row_stride, long col_stride, long pad_rows, long pad_cols,        \
      int precision, void *stream) {                                                          \
    (void)precision;                                                                          \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_spatial_backward", g, batches, input_cols, input_rows, 1,     \
                       in_channel, kernel_cols, kernel_rows, 1, output_cols, output_rows, 1,  \
                       col_stride, row_stride, 1);                                            \
    if (rc) return rc;                                                                        \
    g.pr = pad_rows < 0 ? 0 : (int)pad_rows;                                                  \
    g.pc = pad_cols < 0 ? 0 : (int)pad_cols;                                                  \
    return pool_bwd(dtype_of<T>(), MODE, g, input, output_grad, input_grad,                   \
                    (cudaStream_t)stream);                                                    \
  }

#define POOL3D(KIND, T, WHICH, MODE)                                                            \
  int owl_##KIND##_ndarray_##WHICH##_cuboid(                                                   \
      const T *input, T *output, long batches, long input_cols, long input_rows,              \
      long input_dpts, long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts, \
      long output_cols, long output_rows, long output_dpts, long dpt_stride, long row_stride, \
      long col_stride, long padding) {                                                        \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_cuboid", g, batches, input_cols, input_rows, input_dpts,      \
                       in_channel, kernel_cols, kernel_rows, kernel_dpts, output_cols,        \
                       output_rows, output_dpts, col_stride, row_stride, dpt_stride);         \
    if (rc) return rc;                                                                        \
    if (check_pool_padding(#WHICH, padding)) return kErrInvalid;                              \
    g.pc = fwd_pad(padding, col_stride, output_cols, kernel_cols, input_cols);                \
    g.pr = fwd_pad(padding, row_stride, output_rows, kernel_rows, input_rows);                \
    g.pd = fwd_pad(padding, dpt_stride, output_dpts, kernel_dpts, input_dpts);                \
    return pool_fwd_host<T>(MODE, g, input, output, nullptr);                                 \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_##WHICH##_cuboid(                                                \
      const T *input, T *output, long batches, long input_cols, long input_rows,              \
      long input_dpts, long in_channel, long kernel_cols, long kernel_rows, long kernel_dpts, \
      long output_cols, long output_rows, long output_dpts, long dpt_stride, long row_stride, \
      long col_stride, long padding, int precision, void *stream) {                           \
    (void)precision;                                                                          \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_cuboid", g, batches, input_cols, input_rows, input_dpts,      \
                       in_channel, kernel_cols, kernel_rows, kernel_dpts, output_cols,        \
                       output_rows, output_dpts, col_stride, row_stride, dpt_stride);         \
    if (rc) return rc;                                                                        \
    if (check_pool_padding(#WHICH, padding)) return kErrInvalid;                              \
    g.pc = fwd_pad(padding, col_stride, output_cols, kernel_cols, input_cols);                \
    g.pr = fwd_pad(padding, row_stride, output_rows, kernel_rows, input_rows);                \
    g.pd = fwd_pad(padding, dpt_stride, output_dpts, kernel_dpts, input_dpts);                \
    return pool_fwd(dtype_of<T>(), MODE, g, input, output, nullptr, (cudaStream_t)stream);    \
  }                                                                                           \
  int owl_##KIND##_ndarray_##WHICH##_cuboid_backward(                                          \
      const T *input, const T *output_grad, T *input_grad, long batches, long input_cols,     \
      long input_rows, long input_dpts, long in_channel, long kernel_cols, long kernel_rows,   \
      long kernel_dpts, long output_cols, long output_rows, long output_dpts, long col_stride, \
      long row_stride, long dpt_stride, long padding) {                                        \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_cuboid_backward", g, batches, input_cols, input_rows,         \
                       input_dpts, in_channel, kernel_cols, kernel_rows, kernel_dpts,         \
                       output_cols, output_rows, output_dpts, col_stride, row_stride,         \
                       dpt_stride);                                                           \
    if (rc) return rc;                                                                        \
    if (check_pool_padding(#WHICH, padding)) return kErrInvalid;                              \
    g.pc = fwd_pad(padding, col_stride, output_cols, kernel_cols, input_cols);                \
    g.pr = fwd_pad(padding, row_stride, output_rows, kernel_rows, input_rows);                \
    g.pd = fwd_pad(padding, dpt_stride, output_dpts, kernel_dpts, input_dpts);                \
    return pool_bwd_host<T>(MODE, g, input, output_grad, input_grad);                         \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_##WHICH##_cuboid_backward(                                       \
      const T *input, const T *output_grad, T *input_grad, long batches, long input_cols,     \
      long input_rows, long input_dpts, long in_channel, long kernel_cols, long kernel_rows,   \
      long kernel_dpts, long output_cols, long output_rows, long output_dpts, long col_stride, \
      long row_stride, long dpt_stride, long padding, int precision, void *stream) {           \
    (void)precision;                                                                          \
    PoolGeom g;                                                                               \
    int rc = make_pool(#WHICH "_cuboid_backward", g, batches, input_cols, input_rows,         \
                       input_dpts, in_channel, kernel_cols, kernel_rows, kernel_dpts,         \
                       output_cols, output_rows, output_dpts, col_stride, row_stride,         \
                       dpt_stride);                                                           \
    if (rc) return rc;                                                                        \
    if (check_pool_padding(#WHICH, padding)) return kErrInvalid;                              \
    g.pc = fwd_pad(padding, col_stride, output_cols, kernel_cols, input_cols);                \
    g.pr = fwd_pad(padding, row_stride, output_rows, kernel_rows, input_rows);                \
    g.pd = fwd_pad(padding, dpt_stride, output_dpts, kernel_dpts, input_dpts);                \
    return pool_bwd(dtype_of<T>(), MODE, g, input, output_grad, input_grad,                   \
                    (cudaStream_t)stream);                                                    \
  }

#define ARGMAX(KIND, T)                                                                         \
  int owl_##KIND##_ndarray_maxpool_argmax_spatial(                                             \
      const T *input, T *output, int64_t *argmax, long batches, long input_cols,              \
      long input_rows, long in_channel, long kernel_cols, long kernel_rows, long output_cols, \
      long output_rows, long row_stride, long col_stride, long pad_rows, long pad_cols) {      \
    PoolGeom g;                                                                               \
    int rc = make_pool("maxpool_argmax_spatial", g, batches, input_cols, input_rows, 1,       \
                       in_channel, kernel_cols, kernel_rows, 1, output_cols, output_rows, 1,  \
                       col_stride, row_stride, 1);                                            \
    if (rc) return rc;                                                                        \
    g.pr = pad_rows < 0 ? 0 : (int)pad_rows;                                                  \
    g.pc = pad_cols < 0 ? 0 : (int)pad_cols;                                                  \
    return pool_fwd_host<T>(POOL_MAX, g, input, output, argmax);                              \
  }                                                                                           \
  int owlgpu_##KIND##_ndarray_maxpool_argmax_spatial(                                          \
      const T *input, T *output, int64_t *argmax, long batches, long input_cols,              \
      long input_rows, long in_channel, long kernel_cols, long kernel_rows, long output_cols, \
      long output_rows, long row_stride, long col_stride, long pad_rows, long pad_cols,        \
      int precision, void *stream) {                                                          \
    (void)precision;                                                                          \
    PoolGeom g;                                                                               \
    int rc = make_pool("maxpool_argmax_spatial", g, batches, input_cols, input_rows, 1,       \
                       in_channel, kernel_cols, kernel_rows, 1, output_cols, output_rows, 1,  \
                       col_stride, row_stride, 1);                                            \
    if (rc) return rc;                                                                        \
    g.pr = pad_rows < 0 ? 0 : (int)pad_rows;                                                  \
    g.pc = pad_cols < 0 ? 0 : (int)pad_cols;                                                  \
    return pool_fwd(dtype_of<T>(), POOL_MAX, g, input, output, argmax, (cudaStream_t)stream); \
  }

#define POOL_ALL(KIND, T)            \
  POOL2D_FWD(KIND, T, maxpool, POOL_MAX) \
  POOL2D_FWD(KIND, T, avgpool, POOL_AVG) \
  POOL2D_BWD(KIND, T, maxpool, POOL_MAX) \
  POOL2D_BWD(KIND, T, avgpool, POOL_AVG) \
  POOL3D(KIND, T, maxpool, POOL_MAX)     \
  POOL3D(KIND, T, avgpool, POOL_AVG)     \
  ARGMAX(KIND, T)

POOL_ALL(float32, float)
POOL_ALL(float64, double)
POOL_ALL(complex32, owlgpu_complex32)
POOL_ALL(complex64, owlgpu_complex64)

// Upsampling: the backward keeps the stub's argument order (input_grad
// written first, then output_grad); the forward, which Owl computes with
// repeat in OCaml, takes the same geometry.
#define UPSAMPLE(KIND, T)                                                                     \
  int owl_##KIND##_ndarray_upsampling_spatial_backward(                                      \
      T *input_grad, const T *output_grad, long batches, long input_cols, long input_rows,   \
      long in_channel, long output_cols, long output_rows, long col_scale, long row_scale) { \
    UpGeom g;                                                                               \
    int rc = make_up("upsampling_spatial_backward", g, false, batches, input_cols,          \
                     input_rows, in_channel, output_cols, output_rows, col_scale, row_scale); \
    if (rc) return rc;                                                                      \
    return up_host<T>(false, g, output_grad, input_grad);                                   \
  }                                                                                         \
  int owlgpu_##KIND##_ndarray_upsampling_spatial_backward(                                   \
      T *input_grad, const T *output_grad, long batches, long input_cols, long input_rows,   \
      long in_channel, long output_cols, long output_rows, long col_scale, long row_scale,   \
      int precision, void *stream) {                                                        \
    (void)precision;                                                                        \
    UpGeom g;                                                                               \
    int rc = make_up("upsampling_spatial_backward", g, false, batches, input_cols,          \
                     input_rows, in_channel, output_cols, output_rows, col_scale, row_scale); \
    if (rc) return rc;                                                                      \
    return upsample_bwd(dtype_of<T>(), g, input_grad, output_grad, (cudaStream_t)stream);   \
  }                                                                                         \
  int owl_##KIND##_ndarray_upsampling_spatial(                                               \
      const T *input, T *output, long batches, long input_cols, long input_rows,            \
      long in_channel, long output_cols, long output_rows, long col_scale, long row_scale) { \
    UpGeom g;                                                                               \
    int rc = make_up("upsampling_spatial", g, true, batches, input_cols, input_rows,        \
                     in_channel, output_cols, output_rows, col_scale, row_scale);           \
    if (rc) return rc;                                                                      \
    return up_host<T>(true, g, input, output);                                              \
  }                                                                                         \
  int owlgpu_##KIND##_ndarray_upsampling_spatial(                                            \
      const T *input, T *output, long batches, long input_cols, long input_rows,            \
      long in_channel, long output_cols, long output_rows, long col_scale, long row_scale,  \
      int precision, void *stream) {                                                        \
    (void)precision;                                                                        \
    UpGeom g;                                                                               \
    int rc = make_up("upsampling_spatial", g, true, batches, input_cols, input_rows,        \
                     in_channel, output_cols, output_rows, col_scale, row_scale);           \
    if (rc) return rc;                                                                      \
    return upsample_fwd(dtype_of<T>(), g, input, output, (cudaStream_t)stream);             \
  }

UPSAMPLE(float32, float)
UPSAMPLE(float64, double)
UPSAMPLE(complex32, owlgpu_complex32)
UPSAMPLE(complex64, owlgpu_complex64)

// ---- forward convolution with bias and activation (Conv2D / Conv3D neuron
// followed by an Activation neuron), no Owl stub ---------------------------

#define CONV_BIAS_ACT(KIND, T)                                                                  \
  int owlgpu_##KIND##_ndarray_conv_spatial_bias_act(                                           \
      const T *input, const T *kernel, T *output, long batches, long input_cols,               \
      long input_rows, long in_channel, long kernel_cols, long kernel_rows, long output_cols,   \
      long output_rows, long out_channel, long row_stride, long col_stride, long padding,      \
      long row_in_stride, long col_in_stride, const T *bias, int act, int precision,           \
      void *stream) {                                                                          \
    (void)row_in_stride;                                                                       \
    (void)col_in_stride;                                                                       \
    ConvGeom g;                                                                                \
    int rc = make_conv("conv_spatial_bias_act", g, batches, input_cols, input_rows, 1,        \
                       in_channel, kernel_cols, kernel_rows, 1, output_cols, output_rows, 1,   \
                       out_channel, col_stride, row_stride, 1, 1, 1, 1, false, padding);       \
    if (rc) return rc;                                                                         \
    if (act != OWLGPU_ACT_NONE && act != OWLGPU_ACT_RELU)                                      \
      return invalid("conv_spatial_bias_act", "unknown activation");                          \
    return conv_fwd(dtype_of<T>(), precision, g, input, kernel, output, (cudaStream_t)stream, \
                    bias, act);                                                                \
  }                                                                                            \
  int owlgpu_##KIND##_ndarray_conv_cuboid_bias_act(                                            \
      const T *input, const T *kernel, T *output, long batches, long input_cols,               \
      long input_rows, long input_dpts, long in_channel, long kernel_cols, long kernel_rows,   \
      long kernel_dpts, long output_cols, long output_rows, long output_dpts,                  \
      long out_channel, long dpt_stride, long row_stride, long col_stride, long padding,       \
      const T *bias, int act, int precision, void *stream) {                                   \
    ConvGeom g;                                                                                \
    int rc = make_conv("conv_cuboid_bias_act", g, batches, input_cols, input_rows, input_dpts,\
                       in_channel, kernel_cols, kernel_rows, kernel_dpts, output_cols,         \
                       output_rows, output_dpts, out_channel, col_stride, row_stride,          \
                       dpt_stride, 1, 1, 1, false, padding);                                   \
    if (rc) return rc;                                                                         \
    if (act != OWLGPU_ACT_NONE && act != OWLGPU_ACT_RELU)                                      \
      return invalid("conv_cuboid_bias_act", "unknown activation");                           \
    return conv_fwd(dtype_of<T>(), precision, g, input, kernel, output, (cudaStream_t)stream, \
                    bias, act);                                                                \
  }

CONV_BIAS_ACT(float32, float)
CONV_BIAS_ACT(float64, double)

}  // extern "C"
