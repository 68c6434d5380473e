// filter.cu -- learned window pre-filter: a BF16 dilated 1-D convolution
// network that scores sequence windows ahead of the CYK stage.
//
// Architecture (fixed): windows of 2W residues (stride W, so every hit of
// length <= W lies inside the first-half-start window), one-hot ACGU input,
// six convolutions of kernel 9 with dilations 1, 2, 4, 8, 16, 32 (4 -> 128
// channels, then 128 -> 128), ReLU after each, max-pool over the window's
// positions, a linear 128 -> 1 read-out.  Each window is zero-padded at its
// ends, as the training network's 'same' padding.  Weights and activations
// are BF16, accumulation FP32.
//
// Layout in HBM: activations [nwin][LP][128] bf16 with LP = 2W rounded up to
// the 128-row tile (rows >= 2W hold zeros); layer 0 weights [9][4][128] f32
// (a gather: the input is one-hot); layers 1-5 weights [5][9][128 co][128 ci]
// bf16, biases [6][128] f32, read-out [128] + 1 f32.
//
// Layers 1-5 are implicit GEMMs (M = window positions, N = 128 output
// channels, K = 9 taps x 128 input channels) on the fifth-generation tensor
// cores (tcgen05.mma, BF16 x BF16 -> FP32 in TMEM): a CTA computes a 128 x 128
// output tile; its input rows for all nine taps (128 + 8 d rows) are staged
// once in shared memory, the tap's weights per tap.
#ifdef CMGB_HOST_EMULATION
#include "cmgb_emu.h"
#endif
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/infernal_gb300.h"

#define FERR(code, ...) do { if (errbuf) snprintf(errbuf, CMGB_ERRBUFSIZE, __VA_ARGS__); return (code); } while (0)
#define FCUDA(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) FERR(CMGB_ENODEV, "CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); } while (0)

namespace {
constexpr int CH = 128;      // channels
constexpr int KT = 9;        // kernel taps
constexpr int NL = 6;        // layers
constexpr int TILE = 128;    // positions per CTA tile
constexpr int DIL[NL] = {1, 2, 4, 8, 16, 32};
}

struct cmgb_filter_s {
  int W = 0, LP = 0;
  float *d_w0 = nullptr;              // [9][4][128]
  unsigned short *d_w = nullptr;      // [5][9][128][128] bf16 bits
  float *d_b = nullptr;               // [6][128]
  float *d_out = nullptr;             // [129]
  unsigned short *d_act[2] = {nullptr, nullptr};
  size_t act_rows = 0;
  float *d_logit = nullptr; size_t logit_n = 0;
  int *d_err = nullptr;               // set by a tensor-core wait that ran out
};

#ifndef CMGB_HOST_EMULATION
__device__ __forceinline__ unsigned short f2bf(float x)
{
  // round to nearest even on the bit pattern (finite inputs)
  unsigned u = __float_as_uint(x);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (unsigned short) (u >> 16);
}
__device__ __forceinline__ float bf2f(unsigned short h) { return __uint_as_float(((unsigned) h) << 16); }

// Layer 0: one-hot input -> 128 channels (a gather of nine weight rows).
__global__ void filter_layer0(const unsigned char *dsq, long long i0, long long j0, long long W, int nwin, int LP,
                              const float *w0, const float *b, unsigned short *out)
{
  const int win = blockIdx.y;
  const int co = threadIdx.x;                  // 128 threads
  const long long ws = i0 + (long long) win * W;   // first residue of the window
  for (int i = blockIdx.x; i < LP; i += gridDim.x) {
    float acc = b[co];
    if (i < 2 * W) {
      for (int t = 0; t < KT; t++) {
        const int q = i + t - 4;
        if (q < 0 || q >= 2 * W) continue;
        const long long pos = ws + q;
        if (pos > j0) continue;
        const int x = dsq[pos];
        if (x < 4) acc += w0[(t * 4 + x) * CH + co];
      }
      acc = acc > 0.f ? acc : 0.f;
    } else acc = 0.f;
    out[((size_t) win * LP + i) * CH + co] = f2bf(acc);
  }
}

// ---- layers 1-5 on tcgen05 ------------------------------------------------
// One CTA (4 warps) computes a 128-position x 128-channel tile with
// tcgen05.mma (cta_group::1, kind::f16, BF16 x BF16 -> FP32, M = N = 128,
// K = 16 per instruction) accumulating in 128 TMEM columns.  Operands sit in
// shared memory in the K-major, non-swizzled canonical layout: 8-row x
// 16-byte core matrices, chunk c (8 input channels) of row r at
// (c * rows + r) * 16 bytes, so a tap's shift by (t * dil) rows is a 16-byte
// multiple of the start address.  Descriptors: leading (K) byte offset =
// one chunk plane, stride (M/N) byte offset = 128 bytes between 8-row core
// matrices.  Thread 0 issues the 8 MMAs of a tap and commits them to an
// mbarrier; every wait is bounded and sets *err on expiry.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned) __cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long umma_desc(unsigned saddr, unsigned lbo, unsigned sbo)
{
  return (unsigned long long) ((saddr >> 4) & 0x3FFFu) | ((unsigned long long) ((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long) ((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);   // version 1, no swizzle
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *mb, unsigned parity)
{
  for (int it = 0; it < (1 << 24); it++) {
    unsigned ok;
    asm volatile("{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n selp.b32 %0, 1, 0, P1;\n}"
                 : "=r"(ok) : "r"(smem_u32(mb)), "r"(parity) : "memory");
    if (ok) return true;
  }
  return false;
}

__global__ void __launch_bounds__(128, 1) filter_conv_tc(const unsigned short *in, unsigned short *out, int LP, int W2, int dil,
                                                         const unsigned short *wt, const float *bias, int *err)
{
  extern __shared__ __align__(1024) unsigned char tsm[];
  const int rows = TILE + 8 * dil;
  unsigned char *sA = tsm;                                    // [16 chunks][rows][16 B]
  unsigned char *sB = tsm + (size_t) 16 * rows * 16;          // [16 chunks][128][16 B]
  unsigned long long *mbar = reinterpret_cast<unsigned long long *>(sB + 16 * CH * 16);
  unsigned *tslot = reinterpret_cast<unsigned *>(mbar + 1);
  const int tile = blockIdx.x, win = blockIdx.y;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(tslot)), "r"(128) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(mbar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const int p0 = tile * TILE - 4 * dil;
  const unsigned short *inw = in + (size_t) win * LP * CH;
  for (int x = tid; x < rows * 16; x += blockDim.x) {
    const int r = x >> 4, c = x & 15;
    const int p = p0 + r;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (p >= 0 && p < LP) v = *reinterpret_cast<const uint4 *>(inw + (size_t) p * CH + c * 8);
    *reinterpret_cast<uint4 *>(sA + ((size_t) c * rows + r) * 16) = v;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned taddr = *tslot;
  // instruction descriptor: D f32, A/B bf16, both K-major, N = 128, M = 128
  const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned) (CH >> 3) << 17) | ((unsigned) (TILE >> 4) << 24);
  bool ok = true;
  for (int t = 0; t < KT && ok; t++) {
    const unsigned short *wtt = wt + (size_t) t * CH * CH;
    for (int x = tid; x < CH * 16; x += blockDim.x) {
      const int co = x >> 4, c = x & 15;
      *reinterpret_cast<uint4 *>(sB + ((size_t) c * CH + co) * 16) = *reinterpret_cast<const uint4 *>(wtt + (size_t) co * CH + c * 8);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic-proxy stores -> tensor-core reads
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kb = 0; kb < CH / 16; kb++) {
        const unsigned long long ad = umma_desc(smem_u32(sA + ((size_t) (2 * kb) * rows + t * dil) * 16), rows * 16, 128);
        const unsigned long long bd = umma_desc(smem_u32(sB + (size_t) (2 * kb) * CH * 16), CH * 16, 128);
        const unsigned acc = (t > 0 || kb > 0) ? 1u : 0u;
        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                     :: "r"(taddr), "l"(ad), "l"(bd), "r"(idesc), "r"(acc) : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(smem_u32(mbar)) : "memory");
    }
    // the tap's MMAs must finish reading sB before it is overwritten
    if (!mbar_wait_bounded(mbar, (unsigned) (t & 1))) { ok = false; if (tid == 0) atomicOr(err, 1); }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  // epilogue: warp w holds tile rows 32 w .. 32 w + 31 (TMEM lanes), 16 columns per load
  unsigned short *outw = out + (size_t) win * LP * CH;
  const int row = tile * TILE + 32 * warp + lane;
  for (int cb = 0; cb < CH / 16; cb++) {
    unsigned r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr + ((unsigned) (32 * warp) << 16) + (unsigned) (cb * 16)));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    unsigned pk[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int co = cb * 16 + 2 * j;
      float v0 = __uint_as_float(r[2 * j]) + bias[co], v1 = __uint_as_float(r[2 * j + 1]) + bias[co + 1];
      v0 = v0 > 0.f ? v0 : 0.f; v1 = v1 > 0.f ? v1 : 0.f;
      if (row >= W2 || !ok) v0 = v1 = 0.f;
      pk[j] = (unsigned) f2bf(v0) | ((unsigned) f2bf(v1) << 16);
    }
    uint4 *dst = reinterpret_cast<uint4 *>(outw + (size_t) row * CH + cb * 16);
    dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(128) : "memory");
}

// Read-out: max over the window's positions per channel, then the linear layer.
__global__ void filter_readout(const unsigned short *act, int LP, int W2, const float *wout, float *logit)
{
  __shared__ float red[CH];
  const int win = blockIdx.x, co = threadIdx.x;
  const unsigned short *a = act + (size_t) win * LP * CH + co;
  float m = 0.f;   // activations are ReLU outputs (>= 0)
  for (int i = 0; i < W2; i++) { const float v = bf2f(a[(size_t) i * CH]); m = v > m ? v : m; }
  red[co] = m * wout[co];
  __syncthreads();
  for (int s = CH / 2; s > 0; s >>= 1) { if (co < s) red[co] += red[co + s]; __syncthreads(); }
  if (co == 0) logit[win] = red[0] + wout[CH];
}
#endif

extern "C" int cmgb_filter_create(cmgb_ctx *ctx, int W, const float *w0, const uint16_t *w, const float *bias,
                                  const float *wout, cmgb_filter **ret, char *errbuf)
{
  (void) ctx;
  *ret = nullptr;
#ifdef CMGB_HOST_EMULATION
  (void) W; (void) w0; (void) w; (void) bias; (void) wout;
  FERR(CMGB_ENODEV, "filter: not available in the host emulation");
#else
  if (W < 1 || !w0 || !w || !bias || !wout) FERR(CMGB_EINVAL, "filter: invalid arguments");
  std::unique_ptr<cmgb_filter> f(new cmgb_filter);
  f->W = W;
  f->LP = ((2 * W + TILE - 1) / TILE) * TILE;
  FCUDA(cudaMalloc(&f->d_w0, sizeof(float) * KT * 4 * CH));
  FCUDA(cudaMalloc(&f->d_w, sizeof(unsigned short) * 5 * KT * CH * CH));
  FCUDA(cudaMalloc(&f->d_b, sizeof(float) * NL * CH));
  FCUDA(cudaMalloc(&f->d_out, sizeof(float) * (CH + 1)));
  FCUDA(cudaMemcpy(f->d_w0, w0, sizeof(float) * KT * 4 * CH, cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->d_w, w, sizeof(unsigned short) * 5 * KT * CH * CH, cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->d_b, bias, sizeof(float) * NL * CH, cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->d_out, wout, sizeof(float) * (CH + 1), cudaMemcpyHostToDevice));
  FCUDA(cudaMalloc(&f->d_err, sizeof(int)));
  FCUDA(cudaMemset(f->d_err, 0, sizeof(int)));
  const int maxsm = 16 * (TILE + 8 * DIL[NL - 1]) * 16 + 16 * CH * 16 + 64;
  FCUDA(cudaFuncSetAttribute(filter_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm));
  *ret = f.release();
  return CMGB_OK;
#endif
}

extern "C" void cmgb_filter_destroy(cmgb_filter *f)
{
  if (!f) return;
#ifndef CMGB_HOST_EMULATION
  cudaFree(f->d_w0); cudaFree(f->d_w); cudaFree(f->d_b); cudaFree(f->d_out);
  cudaFree(f->d_act[0]); cudaFree(f->d_act[1]); cudaFree(f->d_logit); cudaFree(f->d_err);
#endif
  delete f;
}

extern "C" int cmgb_filter_windows(cmgb_ctx *ctx, cmgb_filter *f, const uint8_t *d_dsq, int64_t i0, int64_t j0,
                                   float *ret_logits, int64_t max_windows, int64_t *ret_nwin, float *ret_ms, char *errbuf)
{
  (void) ctx;
#ifdef CMGB_HOST_EMULATION
  (void) f; (void) d_dsq; (void) i0; (void) j0; (void) ret_logits; (void) max_windows; (void) ret_nwin; (void) ret_ms;
  FERR(CMGB_ENODEV, "filter: not available in the host emulation");
#else
  if (!f || !d_dsq || j0 < i0 || i0 < 1) FERR(CMGB_EINCOMPAT, "filter: invalid range or arguments");
  const int64_t L = j0 - i0 + 1, W = f->W;
  const int64_t nwin64 = (L + W - 1) / W;   // window k covers [i0 + kW, i0 + kW + 2W - 1] (clipped at j0)
  if (nwin64 > max_windows || nwin64 > 65535) FERR(CMGB_ERANGE, "filter: %lld windows exceed the output (%lld) or a launch (65535)",
                                                    (long long) nwin64, (long long) max_windows);
  const int nwin = (int) nwin64;
  const size_t rows = (size_t) nwin * f->LP;
  if (rows > f->act_rows) {
    cudaFree(f->d_act[0]); cudaFree(f->d_act[1]);
    f->d_act[0] = f->d_act[1] = nullptr;
    FCUDA(cudaMalloc(&f->d_act[0], rows * CH * sizeof(unsigned short)));
    FCUDA(cudaMalloc(&f->d_act[1], rows * CH * sizeof(unsigned short)));
    f->act_rows = rows;
  }
  if ((size_t) nwin > f->logit_n) {
    cudaFree(f->d_logit); f->d_logit = nullptr;
    FCUDA(cudaMalloc(&f->d_logit, sizeof(float) * nwin));
    f->logit_n = nwin;
  }
  cudaEvent_t e0, e1;
  FCUDA(cudaEventCreate(&e0)); FCUDA(cudaEventCreate(&e1));
  FCUDA(cudaEventRecord(e0));
  filter_layer0<<<dim3(64, nwin), CH>>>(d_dsq, i0, j0, W, nwin, f->LP, f->d_w0, f->d_b, f->d_act[0]);
  FCUDA(cudaGetLastError());
  int cur = 0;
  for (int l = 1; l < NL; l++) {
    const int d = DIL[l];
    const size_t sm = (size_t) 16 * (TILE + 8 * d) * 16 + (size_t) 16 * CH * 16 + 64;
    filter_conv_tc<<<dim3(f->LP / TILE, nwin), 128, sm>>>(f->d_act[cur], f->d_act[cur ^ 1], f->LP, (int) (2 * W), d,
                                                          f->d_w + (size_t) (l - 1) * KT * CH * CH, f->d_b + l * CH, f->d_err);
    FCUDA(cudaGetLastError());
    cur ^= 1;
  }
  filter_readout<<<nwin, CH>>>(f->d_act[cur], f->LP, (int) (2 * W), f->d_out, f->d_logit);
  FCUDA(cudaGetLastError());
  FCUDA(cudaEventRecord(e1));
  FCUDA(cudaMemcpy(ret_logits, f->d_logit, sizeof(float) * nwin, cudaMemcpyDeviceToHost));
  int herr = 0;
  FCUDA(cudaMemcpy(&herr, f->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) FERR(CMGB_ENODEV, "filter: a bounded tensor-core wait ran out");
  float ms = 0.f;
  FCUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  if (ret_nwin) *ret_nwin = nwin;
  if (ret_ms) *ret_ms = ms;
  return CMGB_OK;
#endif
}
