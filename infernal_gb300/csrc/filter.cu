// filter.cu -- learned window pre-filter: a BF16 dilated 1-D convolution
// network that scores sequence windows ahead of the CYK stage.
//
// Architecture (fixed): windows of 2W residues (stride W, so every hit of
// length <= W lies inside the first-half-start window), one-hot ACGU input,
// six convolutions of kernel 9 with dilations 1, 2, 4, 8, 16, 32 (4 -> 128
// channels, then 128 -> 128), ReLU after each, max-pool over the window's
// positions, a linear 128 -> 1 read-out per head (one head per CM when one
// network filters for several CMs: the convolutions are shared, each CM has
// its own read-out and threshold).  Each window is zero-padded at its ends,
// as the training network's 'same' padding.  Weights and activations are
// BF16, accumulation FP32.
//
// Layout in HBM: activations [nwin][LP][128] bf16 with LP = 2W rounded up to
// the 128-row tile (rows >= 2W hold zeros); layer 0 weights [9][4][128] f32
// (a gather: the input is one-hot); layers 1-5 weights [5][9][128 co][128 ci]
// bf16, biases [6][128] f32, read-out [heads][128 + 1] f32.
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
  int W = 0, LP = 0, H = 1;           // H: read-out heads
  float *d_w0 = nullptr;              // [9][4][128]
  unsigned short *d_w = nullptr;      // [5][9][128][128] bf16 bits
  float *d_b = nullptr;               // [6][128]
  float *d_out = nullptr;             // [H][129]
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
// Window win starts at residue i0 + win * wstride (W when scanning, 2W for
// training batches stored back to back).  A block computes one 128-row tile
// of one window: the tile's residue codes (and four on each side) and the
// weights sit in shared memory, and each thread produces eight channels of a
// row (one 16-byte store), summing the taps in order.
__global__ void __launch_bounds__(256) filter_layer0(const unsigned char *dsq, long long i0, long long j0, long long W,
                                                     long long wstride, int nwin, int LP, const float *w0, const float *b,
                                                     unsigned short *out)
{
  __shared__ float sw[KT * 4 * CH];
  __shared__ float sb[CH];
  __shared__ unsigned char sx[TILE + KT - 1];
  const int tile = blockIdx.x, win = blockIdx.y;
  const long long ws = i0 + (long long) win * wstride;   // first residue of the window
  for (int k = threadIdx.x; k < KT * 4 * CH; k += blockDim.x) sw[k] = w0[k];
  for (int k = threadIdx.x; k < CH; k += blockDim.x) sb[k] = b[k];
  for (int k = threadIdx.x; k < TILE + KT - 1; k += blockDim.x) {
    const long long q = (long long) tile * TILE + k - 4;   // window position of tap row k
    unsigned char x = 255;
    if (q >= 0 && q < 2 * W && ws + q <= j0) { const unsigned char c = dsq[ws + q]; if (c < 4) x = c; }
    sx[k] = x;
  }
  __syncthreads();
  for (int task = threadIdx.x; task < TILE * (CH / 8); task += blockDim.x) {
    const int r = task / (CH / 8), cg = task % (CH / 8);
    const int i = tile * TILE + r;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (i < 2 * W) {
      float acc[8];
#pragma unroll
      for (int c = 0; c < 8; c++) acc[c] = sb[cg * 8 + c];
      for (int t = 0; t < KT; t++) {
        const unsigned char x = sx[r + t];
        if (x < 4) {
          const float *wr = sw + (t * 4 + x) * CH + cg * 8;
#pragma unroll
          for (int c = 0; c < 8; c++) acc[c] += wr[c];
        }
      }
      unsigned pk[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const float a0 = acc[2 * c] > 0.f ? acc[2 * c] : 0.f, a1 = acc[2 * c + 1] > 0.f ? acc[2 * c + 1] : 0.f;
        pk[c] = (unsigned) f2bf(a0) | ((unsigned) f2bf(a1) << 16);
      }
      v = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
    *reinterpret_cast<uint4 *>(out + ((size_t) win * LP + i) * CH + cg * 8) = v;
  }
}

// ---- layers 1-5 on tcgen05 ------------------------------------------------
// One CTA (4 warps) computes up to TPC 128-position tiles of one window
// against all 128 output channels with tcgen05.mma (cta_group::1, kind::f16,
// BF16 x BF16 -> FP32, M = N = 128, K = 16 per instruction), one TMEM
// accumulator of 128 columns per tile.  Operands sit in shared memory in the
// K-major, non-swizzled canonical layout: 8-row x 16-byte core matrices,
// chunk c (8 input channels) of row r at (c * rows + r) * 16 bytes, so a tap's
// shift by (t * dil) rows is a 16-byte multiple of the start address.
// Descriptors: leading (K) byte offset = one chunk plane, stride (M/N) byte
// offset = 128 bytes between 8-row core matrices.
//
// The input rows of all nine taps are staged once.  The weights are stored
// pre-packed in the same operand layout ([layer][tap][chunk][out channel][8]),
// so a tap is one 32 KB bulk copy (cp.async.bulk) into a ring of NSTG stages:
// thread 0 issues a tap's MMAs (for every tile, sharing the tap's weights) as
// soon as its copy has landed, and refills a stage with the tap NSTG ahead
// once the MMAs reading it have completed (tcgen05.commit to an mbarrier).
// Every wait is bounded and sets *err on expiry.
constexpr int TAP_BYTES = CH * CH * 2;        // one tap's packed weights
// TPC tiles per CTA, NSTG weight stages
__host__ __device__ constexpr size_t conv_smem(int tpc, int nstg, int dil) { return (size_t) 16 * (tpc * TILE + 8 * dil) * 16 + (size_t) nstg * TAP_BYTES + 128; }
// Dilations up to 8 use one tile and two stages per CTA (at most 112 KB, so
// two CTAs share an SM and one's staging and epilogue overlap the other's
// MMAs); wider dilations two tiles and three stages (one CTA per SM).
constexpr bool conv_small(int dil) { return dil <= 8; }

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
// one tap's packed weights: global -> shared stage, completing on mb
__device__ __forceinline__ void tap_copy(void *dst, const void *src, unsigned long long *mb)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(mb)), "r"(TAP_BYTES) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_u32(dst)), "l"(src), "r"(TAP_BYTES), "r"(smem_u32(mb)) : "memory");
}

// mask == NULL: out = bf16(relu(acc + bias)) (a forward layer).  mask != NULL:
// out = bf16(acc) where mask > 0, else 0, no bias (the input gradient of a
// layer, with the previous layer's ReLU derivative folded in).
template <int TPC, int NSTG>
__global__ void __launch_bounds__(128, 1) filter_conv_tc(const unsigned short *in, unsigned short *out, int LP, int W2, int dil,
                                                         const unsigned short *wt, const float *bias, int *err,
                                                         const unsigned short *mask)
{
  extern __shared__ __align__(1024) unsigned char tsm[];
  const int rows = TPC * TILE + 8 * dil;
  unsigned char *sA = tsm;                                    // [16 chunks][rows][16 B]
  unsigned char *sB = tsm + (size_t) 16 * rows * 16;          // [NSTG][16 chunks][128][16 B]
  unsigned long long *mbW = reinterpret_cast<unsigned long long *>(sB + (size_t) NSTG * TAP_BYTES);   // stage's copy landed
  unsigned long long *mbM = mbW + NSTG;                                                              // stage's MMAs done
  unsigned *tslot = reinterpret_cast<unsigned *>(mbM + NSTG);
  int *s_ok = reinterpret_cast<int *>(tslot + 1);   // thread 0's verdict, for the epilogue
  const int tile0 = blockIdx.x * TPC, win = blockIdx.y;
  const int ntile = LP / TILE - tile0 < TPC ? LP / TILE - tile0 : TPC;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(tslot)), "r"(TPC * 128) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  int issued[NSTG] = {0}, landed[NSTG] = {0};   // thread 0: copies issued / waited for, per stage
  if (tid == 0) {
    for (int q = 0; q < 2 * NSTG; q++) asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(mbW + q)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int t = 0; t < NSTG && t < KT; t++) { tap_copy(sB + (size_t) t * TAP_BYTES, wt + (size_t) t * CH * CH, mbW + t); issued[t]++; }
  }
  const int p0 = tile0 * TILE - 4 * dil;
  const unsigned short *inw = in + (size_t) win * LP * CH;
  for (int x = tid; x < rows * 16; x += blockDim.x) {
    const int r = x >> 4, c = x & 15;
    const int p = p0 + r;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (p >= 0 && p < LP) v = *reinterpret_cast<const uint4 *>(inw + (size_t) p * CH + c * 8);
    *reinterpret_cast<uint4 *>(sA + ((size_t) c * rows + r) * 16) = v;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic-proxy stores -> tensor-core reads
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned taddr = *tslot;
  // instruction descriptor: D f32, A/B bf16, both K-major, N = 128, M = 128
  const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned) (CH >> 3) << 17) | ((unsigned) (TILE >> 4) << 24);
  if (tid == 0) {
    bool ok = true;
    int committed = 0;   // taps whose MMAs were committed
    for (int t = 0; t < KT && ok; t++) {
      const int st = t % NSTG;
      ok = mbar_wait_bounded(mbW + st, (unsigned) ((t / NSTG) & 1));
      if (!ok) break;
      landed[st]++;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned char *stg = sB + (size_t) st * TAP_BYTES;
      for (int u = 0; u < ntile; u++)
        for (int kb = 0; kb < CH / 16; kb++) {
          const unsigned long long ad = umma_desc(smem_u32(sA + ((size_t) (2 * kb) * rows + u * TILE + t * dil) * 16), rows * 16, 128);
          const unsigned long long bd = umma_desc(smem_u32(stg + (size_t) (2 * kb) * CH * 16), CH * 16, 128);
          const unsigned acc = (t > 0 || kb > 0) ? 1u : 0u;
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                       :: "r"(taddr + (unsigned) (u * 128)), "l"(ad), "l"(bd), "r"(idesc), "r"(acc) : "memory");
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(smem_u32(mbM + st)) : "memory");
      committed = t + 1;
      // refill the previous tap's stage with the tap NSTG after it, once its MMAs are done
      if (t >= 1 && t - 1 + NSTG < KT) {
        const int sp = (t - 1) % NSTG;
        ok = mbar_wait_bounded(mbM + sp, (unsigned) (((t - 1) / NSTG) & 1));
        if (!ok) break;
        tap_copy(sB + (size_t) sp * TAP_BYTES, wt + (size_t) (t - 1 + NSTG) * CH * CH, mbW + sp);
        issued[sp]++;
      }
    }
    // the MMAs complete in order: the last tap's commit means all are done
    if (ok) ok = mbar_wait_bounded(mbM + (KT - 1) % NSTG, (unsigned) (((KT - 1) / NSTG) & 1));
    if (!ok) {
      atomicOr(err, 1);
      // let the committed MMAs finish (they complete in order) and every
      // weight copy still in flight land before TMEM is freed and the CTA exits
      if (committed > 0) mbar_wait_bounded(mbM + (committed - 1) % NSTG, (unsigned) (((committed - 1) / NSTG) & 1));
      for (int q = 0; q < NSTG; q++)
        while (landed[q] < issued[q]) { mbar_wait_bounded(mbW + q, (unsigned) (landed[q] & 1)); landed[q]++; }
    }
    *s_ok = ok ? 1 : 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool ok = *s_ok != 0;
  // epilogue: warp w holds tile rows 32 w .. 32 w + 31 (TMEM lanes), 16 columns per load
  unsigned short *outw = out + (size_t) win * LP * CH;
  for (int u = 0; u < ntile; u++) {
    const int row = (tile0 + u) * TILE + 32 * warp + lane;
    for (int cb = 0; cb < CH / 16; cb++) {
      unsigned r[16];
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                     "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                   : "r"(taddr + ((unsigned) (32 * warp) << 16) + (unsigned) (u * 128 + cb * 16)));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      unsigned pk[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int co = cb * 16 + 2 * j;
        float v0, v1;
        if (mask) {
          const unsigned mk = *reinterpret_cast<const unsigned *>(mask + (size_t) win * LP * CH + (size_t) row * CH + co);
          v0 = (mk & 0xFFFFu) != 0 ? __uint_as_float(r[2 * j]) : 0.f;      // activations are >= 0: nonzero bits <=> > 0
          v1 = (mk >> 16) != 0 ? __uint_as_float(r[2 * j + 1]) : 0.f;
        } else {
          v0 = __uint_as_float(r[2 * j]) + bias[co]; v1 = __uint_as_float(r[2 * j + 1]) + bias[co + 1];
          v0 = v0 > 0.f ? v0 : 0.f; v1 = v1 > 0.f ? v1 : 0.f;
        }
        if (row >= W2 || !ok) v0 = v1 = 0.f;
        pk[j] = (unsigned) f2bf(v0) | ((unsigned) f2bf(v1) << 16);
      }
      uint4 *dst = reinterpret_cast<uint4 *>(outw + (size_t) row * CH + cb * 16);
      dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(TPC * 128) : "memory");
}

// One dilated layer over LP/TILE tiles of nwin windows.
static cudaError_t conv_launch(const unsigned short *in, unsigned short *out, int LP, int W2, int dil, int nwin,
                               const unsigned short *wt, const float *bias, int *err, const unsigned short *mask)
{
  const int ntile = LP / TILE;
  if (conv_small(dil))
    filter_conv_tc<1, 2><<<dim3(ntile, nwin), 128, conv_smem(1, 2, dil)>>>(in, out, LP, W2, dil, wt, bias, err, mask);
  else
    filter_conv_tc<2, 3><<<dim3((ntile + 1) / 2, nwin), 128, conv_smem(2, 3, dil)>>>(in, out, LP, W2, dil, wt, bias, err, mask);
  return cudaGetLastError();
}
static cudaError_t conv_prepare()
{
  cudaError_t e = cudaFuncSetAttribute(filter_conv_tc<1, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) conv_smem(1, 2, 8));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(filter_conv_tc<2, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) conv_smem(2, 3, DIL[NL - 1]));
  return e;
}

// Packs dilated-layer weights [l][t][co][ci] (bf16 bits) into the operand
// layout [l][t][ci / 8][co][ci % 8] that one bulk copy per tap stages.
static void pack_conv_weights(const uint16_t *w, std::vector<uint16_t> &pk)
{
  pk.assign((size_t) 5 * KT * CH * CH, 0);
  for (int lt = 0; lt < 5 * KT; lt++)
    for (int co = 0; co < CH; co++)
      for (int ci = 0; ci < CH; ci++)
        pk[(((size_t) lt * 16 + ci / 8) * CH + co) * 8 + ci % 8] = w[((size_t) lt * CH + co) * CH + ci];
}

// Read-out: max over the window's positions per channel, then each head's
// linear layer (logit[win][h]; the same tree sum per head).
__global__ void filter_readout(const unsigned short *act, int LP, int W2, const float *wout, int H, float *logit)
{
  __shared__ float red[CH];
  const int win = blockIdx.x, co = threadIdx.x;
  const unsigned short *a = act + (size_t) win * LP * CH + co;
  float m = 0.f;   // activations are ReLU outputs (>= 0)
  for (int i = 0; i < W2; i++) { const float v = bf2f(a[(size_t) i * CH]); m = v > m ? v : m; }
  for (int h = 0; h < H; h++) {
    const float *wo = wout + (size_t) h * (CH + 1);
    red[co] = m * wo[co];
    __syncthreads();
    for (int s = CH / 2; s > 0; s >>= 1) { if (co < s) red[co] += red[co + s]; __syncthreads(); }
    if (co == 0) logit[(size_t) win * H + h] = red[0] + wo[CH];
    __syncthreads();
  }
}
#endif

extern "C" int cmgb_filter_create_heads(cmgb_ctx *ctx, int W, int nheads, const float *w0, const uint16_t *w,
                                        const float *bias, const float *wout, cmgb_filter **ret, char *errbuf)
{
  (void) ctx;
  *ret = nullptr;
#ifdef CMGB_HOST_EMULATION
  (void) W; (void) nheads; (void) w0; (void) w; (void) bias; (void) wout;
  FERR(CMGB_ENODEV, "filter: not available in the host emulation");
#else
  if (W < 1 || nheads < 1 || nheads > CMGB_FILTER_MAX_HEADS || !w0 || !w || !bias || !wout)
    FERR(CMGB_EINVAL, "filter: invalid arguments");
  std::unique_ptr<cmgb_filter> f(new cmgb_filter);
  f->W = W; f->H = nheads;
  f->LP = ((2 * W + TILE - 1) / TILE) * TILE;
  FCUDA(cudaMalloc(&f->d_w0, sizeof(float) * KT * 4 * CH));
  FCUDA(cudaMalloc(&f->d_w, sizeof(unsigned short) * 5 * KT * CH * CH));
  FCUDA(cudaMalloc(&f->d_b, sizeof(float) * NL * CH));
  FCUDA(cudaMalloc(&f->d_out, sizeof(float) * (CH + 1) * nheads));
  FCUDA(cudaMemcpy(f->d_w0, w0, sizeof(float) * KT * 4 * CH, cudaMemcpyHostToDevice));
  {
    std::vector<uint16_t> pk;
    pack_conv_weights(w, pk);
    FCUDA(cudaMemcpy(f->d_w, pk.data(), sizeof(unsigned short) * 5 * KT * CH * CH, cudaMemcpyHostToDevice));
  }
  FCUDA(cudaMemcpy(f->d_b, bias, sizeof(float) * NL * CH, cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->d_out, wout, sizeof(float) * (CH + 1) * nheads, cudaMemcpyHostToDevice));
  FCUDA(cudaMalloc(&f->d_err, sizeof(int)));
  FCUDA(cudaMemset(f->d_err, 0, sizeof(int)));
  FCUDA(conv_prepare());
  *ret = f.release();
  return CMGB_OK;
#endif
}

extern "C" int cmgb_filter_create(cmgb_ctx *ctx, int W, const float *w0, const uint16_t *w, const float *bias,
                                  const float *wout, cmgb_filter **ret, char *errbuf)
{
  return cmgb_filter_create_heads(ctx, W, 1, w0, w, bias, wout, ret, errbuf);
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
  if ((size_t) nwin * f->H > f->logit_n) {
    cudaFree(f->d_logit); f->d_logit = nullptr;
    FCUDA(cudaMalloc(&f->d_logit, sizeof(float) * nwin * f->H));
    f->logit_n = (size_t) nwin * f->H;
  }
  cudaEvent_t e0, e1;
  FCUDA(cudaEventCreate(&e0)); FCUDA(cudaEventCreate(&e1));
  FCUDA(cudaEventRecord(e0));
  filter_layer0<<<dim3(f->LP / TILE, nwin), 256>>>(d_dsq, i0, j0, W, W, nwin, f->LP, f->d_w0, f->d_b, f->d_act[0]);
  FCUDA(cudaGetLastError());
  int cur = 0;
  for (int l = 1; l < NL; l++) {
    const int d = DIL[l];
    FCUDA(conv_launch(f->d_act[cur], f->d_act[cur ^ 1], f->LP, (int) (2 * W), d, nwin, f->d_w + (size_t) (l - 1) * KT * CH * CH,
                      f->d_b + l * CH, f->d_err, nullptr));
    FCUDA(cudaGetLastError());
    cur ^= 1;
  }
  filter_readout<<<nwin, CH>>>(f->d_act[cur], f->LP, (int) (2 * W), f->d_out, f->H, f->d_logit);
  FCUDA(cudaGetLastError());
  FCUDA(cudaEventRecord(e1));
  FCUDA(cudaMemcpy(ret_logits, f->d_logit, sizeof(float) * nwin * f->H, cudaMemcpyDeviceToHost));
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

// ---------------------------------------------------------------------------
// Training.  The network above without batch normalisation (convolution,
// bias, ReLU), trained on batches of B windows of 2W residues with a
// pos-weighted logistic loss and AdamW, all on the device:
//   forward   layer 0 gather, layers 1-5 on tcgen05 (every activation kept),
//             max over positions (arg-max kept), linear read-out, loss;
//   backward  read-out -> the arg-max cells of layer 5; per layer l = 5..1:
//             bias gradient (column sums), weight gradient (CUDA-core
//             reduction over every position, fp32), input gradient on
//             tcgen05 as a forward convolution with the taps reversed and
//             each tap's weights transposed, the ReLU derivative of layer
//             l-1 folded into its epilogue; layer 0's weight gradient is a
//             scatter over the one-hot residues;
//   update    AdamW on fp32 master weights, then BF16 copies for the
//             forward and (transposed, taps reversed) for the backward.
// Gradients of a layer's input are rounded to BF16 (the tensor-core
// operand type); weight and bias gradients accumulate in fp32.
//
// Every reduction is deterministic: a block writes its partial sums to its
// own slot of a partial buffer and a second kernel adds the slots in a fixed
// order (no floating-point atomics), so two runs from the same seed on the
// same batches give bit-identical losses and weights.
namespace {
constexpr int NB_BIAS = 256;   // partial slots of a bias gradient (row-strided blocks)
constexpr int NB_W0 = 128;     // partial slots of layer 0's weight gradient (position slices)
constexpr size_t OFF_W0 = 0;                                   // [9][4][128]
constexpr size_t OFF_W = OFF_W0 + (size_t) KT * 4 * CH;        // [5][9][128 co][128 ci]
constexpr size_t OFF_B = OFF_W + (size_t) 5 * KT * CH * CH;    // [6][128]
constexpr size_t OFF_WOUT = OFF_B + (size_t) NL * CH;          // [heads][128 + bias]
inline size_t nparam(int H) { return OFF_WOUT + (size_t) H * (CH + 1); }
}

struct cmgb_filter_trainer_s {
  int W = 0, LP = 0, B = 0, H = 1;                  // H: read-out heads
  size_t np = 0;                                    // parameters
  float *posw = nullptr;                            // [H] positive-class weights
  long long t = 0;                                  // AdamW steps taken
  float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;   // [np] each
  unsigned short *wbf = nullptr, *wtbf = nullptr;   // [5][9][128][128]
  unsigned char *win = nullptr;                     // [B][2W]
  float *y = nullptr, *pooled = nullptr, *logit = nullptr, *dlogit = nullptr, *loss = nullptr;   // y, logit, dlogit: [B][H]
  int *argm = nullptr;
  unsigned short *act[NL] = {nullptr};              // [B][LP][128]
  unsigned short *dz[2] = {nullptr, nullptr};
  int zsplit = 1;                                   // position slices of a dilated layer's weight gradient
  float *part_w = nullptr;                          // [zsplit][9][128][128] partial weight gradients
  float *part_b = nullptr;                          // [NB_BIAS][128] partial bias gradients
  float *part_w0 = nullptr;                         // [NB_W0][9][4][128] partial layer-0 weight gradients
  int *err = nullptr;
};

#ifndef CMGB_HOST_EMULATION
// max over positions (first arg-max) per channel, then each head's read-out
__global__ void train_readout_fwd(const unsigned short *act, int LP, int W2, const float *wout, int H, float *pooled, int *argm,
                                  float *logit)
{
  __shared__ float red[CH];
  const int b = blockIdx.x, c = threadIdx.x;
  const unsigned short *a = act + (size_t) b * LP * CH + c;
  float m = 0.f; int am = 0;
  for (int i = 0; i < W2; i++) { const float v = bf2f(a[(size_t) i * CH]); if (v > m) { m = v; am = i; } }
  pooled[b * CH + c] = m; argm[b * CH + c] = am;
  for (int h = 0; h < H; h++) {
    const float *wo = wout + (size_t) h * (CH + 1);
    red[c] = m * wo[c];
    __syncthreads();
    for (int s = CH / 2; s > 0; s >>= 1) { if (c < s) red[c] += red[c + s]; __syncthreads(); }
    if (c == 0) logit[(size_t) b * H + h] = red[0] + wo[CH];
    __syncthreads();
  }
}

// loss = (1/B) sum_b sum_h [ -w_h y log s(z) - (1 - y) log(1 - s(z)) ],  dz = d loss / d z
__global__ void train_loss(const float *logit, const float *y, const float *posw_h, int B, int H, float *dlogit, float *loss)
{
  __shared__ float red[256];
  float acc = 0.f;
  for (int q = threadIdx.x; q < B * H; q += blockDim.x) {
    const float z = logit[q], t = y[q], posw = posw_h[q % H];
    const float ls = z >= 0.f ? -log1pf(expf(-z)) : z - log1pf(expf(z));        // log s(z)
    const float l1s = z >= 0.f ? -z - log1pf(expf(-z)) : -log1pf(expf(z));      // log (1 - s(z))
    const float s = 1.f / (1.f + expf(-z));
    acc += -posw * t * ls - (1.f - t) * l1s;
    dlogit[q] = (posw * t * (s - 1.f) + (1.f - t) * s) / (float) B;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) { if ((int) threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s]; __syncthreads(); }
  if (threadIdx.x == 0) *loss = red[0] / (float) B;
}

// out[i] = sum over k = 0, 1, .., nparts - 1 (in that order) of part[k n + i]
__global__ void train_sum_parts(const float *part, int nparts, long long n, float *out)
{
  for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < nparts; k++) s += part[(size_t) k * n + i];
    out[i] = s;
  }
}

// read-out backward: the layer-5 gradient at the arg-max cells (one block
// per window), summed over the heads in head order
__global__ void train_readout_bwd(const float *dlogit, const float *pooled, const int *argm, const float *wout, int H, int LP,
                                  unsigned short *dz5)
{
  const int b = blockIdx.x, c = threadIdx.x;
  const float pv = pooled[b * CH + c];
  float d = dlogit[(size_t) b * H] * wout[c];
  for (int h = 1; h < H; h++) d += dlogit[(size_t) b * H + h] * wout[(size_t) h * (CH + 1) + c];
  if (pv > 0.f) dz5[((size_t) b * LP + argm[b * CH + c]) * CH + c] = f2bf(d);
}

// read-out weight gradients, block h = head: thread c < 128 sums
// dlogit[b][h] * pooled[b][c] over the batch in window order, thread 128 the
// bias term (CH + 1 threads)
__global__ void train_readout_wgrad(const float *dlogit, const float *pooled, int B, int H, float *g_wout)
{
  const int h = blockIdx.x, c = threadIdx.x;
  float s = 0.f;
  if (c < CH) for (int b = 0; b < B; b++) s += dlogit[(size_t) b * H + h] * pooled[(size_t) b * CH + c];
  else for (int b = 0; b < B; b++) s += dlogit[(size_t) b * H + h];
  g_wout[(size_t) h * (CH + 1) + c] = s;
}

// bias gradient, partial: block k sums rows k, k + gridDim.x, .. of dz into part[k][c]
__global__ void train_bias_grad(const unsigned short *dz, long long nrows, float *part)
{
  const int c = threadIdx.x;
  float acc = 0.f;
  for (long long r = blockIdx.x; r < nrows; r += gridDim.x) acc += bf2f(dz[(size_t) r * CH + c]);
  part[(size_t) blockIdx.x * CH + c] = acc;
}

// weight gradient of a dilated layer, partial: part[z][t][co][ci] = sum over
// the (b, p) of position slice z of dz[b][p][co] * a[b][p + (t - 4) dil][ci];
// block: one tap, a 32 x 32 (co, ci) tile, one slice; 256 threads x 2 x 2 outputs
__global__ void __launch_bounds__(256) train_wgrad(const unsigned short *dz, const unsigned short *a, int B, int LP, int W2,
                                                   int dil, float *part)
{
  __shared__ float sd[32][33], sa[32][33];
  const int t = blockIdx.x, co0 = (blockIdx.y >> 2) * 32, ci0 = (blockIdx.y & 3) * 32;
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const long long npos = (long long) B * LP;
  const long long per = (npos + gridDim.z - 1) / gridDim.z;
  const long long P0 = per * blockIdx.z, P1 = P0 + per < npos ? P0 + per : npos;
  const int sh = (t - 4) * dil;
  float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
  for (long long P = P0; P < P1; P += 32) {
    for (int x = tid; x < 32 * 32; x += 256) {
      const int r = x >> 5, c = x & 31;
      const long long Q = P + r;
      float vd = 0.f, va = 0.f;
      if (Q < P1) {
        const int b = (int) (Q / LP), p = (int) (Q - (long long) b * LP);
        if (p < W2) {
          vd = bf2f(dz[(size_t) Q * CH + co0 + c]);
          const int q = p + sh;
          if (q >= 0 && q < W2) va = bf2f(a[((size_t) b * LP + q) * CH + ci0 + c]);
        }
      }
      sd[r][c] = vd; sa[r][c] = va;
    }
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < 32; r++) {
      const float d0 = sd[r][2 * ty], d1 = sd[r][2 * ty + 1], a0 = sa[r][2 * tx], a1 = sa[r][2 * tx + 1];
      acc[0][0] += d0 * a0; acc[0][1] += d0 * a1; acc[1][0] += d1 * a0; acc[1][1] += d1 * a1;
    }
    __syncthreads();
  }
  float *o = part + ((size_t) blockIdx.z * KT + t) * CH * CH;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) o[(size_t) (co0 + 2 * ty + i) * CH + ci0 + 2 * tx + j] = acc[i][j];
}

// layer 0 weight gradient, partial: part[k][t][x][co] = sum of dz0[b][p][co]
// over the positions (b, p) of slice k (of the B x 2W flattened in window
// order) where residue p + t - 4 of window b is x (128 threads = co)
__global__ void train_wgrad0(const unsigned short *dz, const unsigned char *win, int B, int LP, int W2, float *part)
{
  __shared__ float acc[KT * 4][CH];
  const int c = threadIdx.x;
  for (int k = 0; k < KT * 4; k++) acc[k][c] = 0.f;
  const long long npos = (long long) B * W2;
  const long long per = (npos + gridDim.x - 1) / gridDim.x;
  const long long Q0 = per * blockIdx.x, Q1 = Q0 + per < npos ? Q0 + per : npos;
  for (long long Q = Q0; Q < Q1; Q++) {
    const int b = (int) (Q / W2), p = (int) (Q - (long long) b * W2);
    const float gv = bf2f(dz[((size_t) b * LP + p) * CH + c]);
    if (gv == 0.f) continue;
    for (int t = 0; t < KT; t++) {
      const int q = p + t - 4;
      if (q < 0 || q >= W2) continue;
      const int x = win[(size_t) b * W2 + q];
      if (x < 4) acc[t * 4 + x][c] += gv;
    }
  }
  float *o = part + (size_t) blockIdx.x * KT * 4 * CH;
  for (int k = 0; k < KT * 4; k++) o[(size_t) k * CH + c] = acc[k][c];
}

__global__ void train_adamw(float *p, const float *g, float *m1, float *m2, long long n, float lr, float b1, float b2,
                            float eps, float wd, float bc1, float bc2)
{
  for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi, v = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a; m2[i] = v;
    p[i] = p[i] * (1.f - lr * wd) - lr * (a / bc1) / (sqrtf(v / bc2) + eps);
  }
}

// BF16 copies of the dilated layers in the convolution's operand layout
// [l][t][k / 8][n][k % 8] (n: output channel, k: input channel): forward
// (n, k) = (co, ci) of w[l][t][co][ci]; backward tap t' = 8 - t with
// (n, k) = (ci, co)
__global__ void train_pack(const float *w, unsigned short *wbf, unsigned short *wtbf)
{
  const long long n = (long long) 5 * KT * CH * CH;
  for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
    const int ci = (int) (i % CH), co = (int) ((i / CH) % CH), t = (int) ((i / (CH * CH)) % KT), l = (int) (i / ((long long) KT * CH * CH));
    const unsigned short h = f2bf(w[i]);
    wbf[((((size_t) l * KT + t) * 16 + ci / 8) * CH + co) * 8 + ci % 8] = h;
    wtbf[((((size_t) l * KT + (KT - 1 - t)) * 16 + co / 8) * CH + ci) * 8 + co % 8] = h;
  }
}
#endif

extern "C" int cmgb_filter_trainer_create_heads(cmgb_ctx *ctx, int W, int batch, int nheads, uint64_t seed,
                                                cmgb_filter_trainer **ret, char *errbuf)
{
  (void) ctx;
  *ret = nullptr;
#ifdef CMGB_HOST_EMULATION
  (void) W; (void) batch; (void) nheads; (void) seed;
  FERR(CMGB_ENODEV, "filter trainer: not available in the host emulation");
#else
  if (W < 16 || batch < 1 || batch > 65535 || nheads < 1 || nheads > CMGB_FILTER_MAX_HEADS)
    FERR(CMGB_EINVAL, "filter trainer: invalid W, batch or head count");
  std::unique_ptr<cmgb_filter_trainer> f(new cmgb_filter_trainer);
  f->W = W; f->B = batch; f->H = nheads; f->LP = ((2 * W + TILE - 1) / TILE) * TILE;
  f->np = nparam(nheads);
  const size_t NPARAM = f->np;
  const size_t act = (size_t) batch * f->LP * CH * sizeof(unsigned short);
  FCUDA(cudaMalloc(&f->p, NPARAM * sizeof(float))); FCUDA(cudaMalloc(&f->g, NPARAM * sizeof(float)));
  FCUDA(cudaMalloc(&f->m1, NPARAM * sizeof(float))); FCUDA(cudaMalloc(&f->m2, NPARAM * sizeof(float)));
  FCUDA(cudaMemset(f->m1, 0, NPARAM * sizeof(float))); FCUDA(cudaMemset(f->m2, 0, NPARAM * sizeof(float)));
  FCUDA(cudaMalloc(&f->wbf, (size_t) 5 * KT * CH * CH * 2)); FCUDA(cudaMalloc(&f->wtbf, (size_t) 5 * KT * CH * CH * 2));
  FCUDA(cudaMalloc(&f->win, (size_t) batch * 2 * W));
  FCUDA(cudaMalloc(&f->y, sizeof(float) * batch * nheads)); FCUDA(cudaMalloc(&f->pooled, sizeof(float) * batch * CH));
  FCUDA(cudaMalloc(&f->logit, sizeof(float) * batch * nheads)); FCUDA(cudaMalloc(&f->dlogit, sizeof(float) * batch * nheads));
  FCUDA(cudaMalloc(&f->posw, sizeof(float) * nheads));
  FCUDA(cudaMalloc(&f->loss, sizeof(float))); FCUDA(cudaMalloc(&f->argm, sizeof(int) * batch * CH));
  for (int l = 0; l < NL; l++) FCUDA(cudaMalloc(&f->act[l], act));
  FCUDA(cudaMalloc(&f->dz[0], act)); FCUDA(cudaMalloc(&f->dz[1], act));
  f->zsplit = std::max(1, std::min(64, (int) (((long long) batch * f->LP) / 2048)));
  FCUDA(cudaMalloc(&f->part_w, sizeof(float) * (size_t) f->zsplit * KT * CH * CH));
  FCUDA(cudaMalloc(&f->part_b, sizeof(float) * (size_t) NB_BIAS * CH));
  FCUDA(cudaMalloc(&f->part_w0, sizeof(float) * (size_t) NB_W0 * KT * 4 * CH));
  FCUDA(cudaMalloc(&f->err, sizeof(int))); FCUDA(cudaMemset(f->err, 0, sizeof(int)));
  // He-uniform initial weights from a splitmix64 stream, zero biases
  std::vector<float> h(NPARAM, 0.f);
  uint64_t s = seed ^ 0x9E3779B97F4A7C15ULL;
  auto uni = [&s]() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL; z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL; z ^= z >> 31;
    return (double) (z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  const double a0 = std::sqrt(6.0 / (4 * KT)), a1 = std::sqrt(6.0 / (CH * KT)), a2 = std::sqrt(6.0 / CH);
  for (size_t i = OFF_W0; i < OFF_W; i++) h[i] = (float) (a0 * uni());
  for (size_t i = OFF_W; i < OFF_B; i++) h[i] = (float) (a1 * uni());
  for (int hd = 0; hd < nheads; hd++)
    for (size_t i = OFF_WOUT + (size_t) hd * (CH + 1); i < OFF_WOUT + (size_t) hd * (CH + 1) + CH; i++) h[i] = (float) (a2 * uni());
  FCUDA(cudaMemcpy(f->p, h.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  train_pack<<<512, 256>>>(f->p + OFF_W, f->wbf, f->wtbf);
  FCUDA(cudaGetLastError());
  FCUDA(conv_prepare());
  FCUDA(cudaDeviceSynchronize());
  *ret = f.release();
  return CMGB_OK;
#endif
}

extern "C" int cmgb_filter_trainer_create(cmgb_ctx *ctx, int W, int batch, uint64_t seed, cmgb_filter_trainer **ret, char *errbuf)
{
  return cmgb_filter_trainer_create_heads(ctx, W, batch, 1, seed, ret, errbuf);
}

extern "C" void cmgb_filter_trainer_destroy(cmgb_filter_trainer *f)
{
  if (!f) return;
#ifndef CMGB_HOST_EMULATION
  cudaFree(f->p); cudaFree(f->g); cudaFree(f->m1); cudaFree(f->m2); cudaFree(f->wbf); cudaFree(f->wtbf);
  cudaFree(f->win); cudaFree(f->y); cudaFree(f->pooled); cudaFree(f->logit); cudaFree(f->dlogit); cudaFree(f->loss);
  cudaFree(f->argm); for (int l = 0; l < NL; l++) cudaFree(f->act[l]);
  cudaFree(f->dz[0]); cudaFree(f->dz[1]); cudaFree(f->err);
  cudaFree(f->part_w); cudaFree(f->part_b); cudaFree(f->part_w0); cudaFree(f->posw);
#endif
  delete f;
}

// Sets the fp32 master weights (layout of cmgb_filter_create, but the dilated
// layers in fp32) and resets the optimiser state.
extern "C" int cmgb_filter_trainer_set(cmgb_filter_trainer *f, const float *w0, const float *w, const float *bias,
                                       const float *wout, char *errbuf)
{
#ifdef CMGB_HOST_EMULATION
  (void) f; (void) w0; (void) w; (void) bias; (void) wout;
  FERR(CMGB_ENODEV, "filter trainer: not available in the host emulation");
#else
  if (!f || !w0 || !w || !bias || !wout) FERR(CMGB_EINVAL, "filter trainer: invalid arguments");
  FCUDA(cudaMemcpy(f->p + OFF_W0, w0, sizeof(float) * (OFF_W - OFF_W0), cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->p + OFF_W, w, sizeof(float) * (OFF_B - OFF_W), cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->p + OFF_B, bias, sizeof(float) * (OFF_WOUT - OFF_B), cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->p + OFF_WOUT, wout, sizeof(float) * (CH + 1) * f->H, cudaMemcpyHostToDevice));
  FCUDA(cudaMemset(f->m1, 0, f->np * sizeof(float))); FCUDA(cudaMemset(f->m2, 0, f->np * sizeof(float)));
  f->t = 0;
  train_pack<<<512, 256>>>(f->p + OFF_W, f->wbf, f->wtbf);
  FCUDA(cudaGetLastError());
  return CMGB_OK;
#endif
}

// One step on a batch: windows (host, [batch][2W] residue codes 0-3, others
// read as missing), labels (host, [batch] 0/1), the positive-class weight and
// the learning rate (0: gradients only, no update).
extern "C" int cmgb_filter_trainer_step_heads(cmgb_filter_trainer *f, const uint8_t *windows, const float *labels,
                                              const float *pos_weights, float lr, float weight_decay, float *ret_loss,
                                              float *ret_ms, char *errbuf)
{
#ifdef CMGB_HOST_EMULATION
  (void) f; (void) windows; (void) labels; (void) pos_weights; (void) lr; (void) weight_decay; (void) ret_loss; (void) ret_ms;
  FERR(CMGB_ENODEV, "filter trainer: not available in the host emulation");
#else
  if (!f || !windows || !labels || !pos_weights) FERR(CMGB_EINVAL, "filter trainer: invalid arguments");
  const int B = f->B, W = f->W, LP = f->LP, W2 = 2 * W, H = f->H;
  const size_t NPARAM = f->np;
  const size_t actb = (size_t) B * LP * CH * sizeof(unsigned short);
  cudaEvent_t e0, e1;
  FCUDA(cudaEventCreate(&e0)); FCUDA(cudaEventCreate(&e1));
  FCUDA(cudaMemcpy(f->win, windows, (size_t) B * W2, cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->y, labels, sizeof(float) * B * H, cudaMemcpyHostToDevice));
  FCUDA(cudaMemcpy(f->posw, pos_weights, sizeof(float) * H, cudaMemcpyHostToDevice));
  FCUDA(cudaEventRecord(e0));
  // forward
  filter_layer0<<<dim3(LP / TILE, B), 256>>>(f->win, 0, (long long) B * W2 - 1, W, W2, B, LP, f->p + OFF_W0, f->p + OFF_B, f->act[0]);
  for (int l = 1; l < NL; l++) {
    const int d = DIL[l];
    conv_launch(f->act[l - 1], f->act[l], LP, W2, d, B, f->wbf + (size_t) (l - 1) * KT * CH * CH, f->p + OFF_B + l * CH, f->err, nullptr);
  }
  train_readout_fwd<<<B, CH>>>(f->act[NL - 1], LP, W2, f->p + OFF_WOUT, H, f->pooled, f->argm, f->logit);
  train_loss<<<1, 256>>>(f->logit, f->y, f->posw, B, H, f->dlogit, f->loss);
  // backward
  FCUDA(cudaMemset(f->g, 0, NPARAM * sizeof(float)));
  FCUDA(cudaMemset(f->dz[0], 0, actb));
  train_readout_bwd<<<B, CH>>>(f->dlogit, f->pooled, f->argm, f->p + OFF_WOUT, H, LP, f->dz[0]);
  train_readout_wgrad<<<H, CH + 1>>>(f->dlogit, f->pooled, B, H, f->g + OFF_WOUT);
  int cur = 0;
  const long long nw = (long long) KT * CH * CH;
  for (int l = NL - 1; l >= 1; l--) {
    const int d = DIL[l];
    train_bias_grad<<<NB_BIAS, CH>>>(f->dz[cur], (long long) B * LP, f->part_b);
    train_sum_parts<<<1, CH>>>(f->part_b, NB_BIAS, CH, f->g + OFF_B + l * CH);
    train_wgrad<<<dim3(KT, 16, f->zsplit), 256>>>(f->dz[cur], f->act[l - 1], B, LP, W2, d, f->part_w);
    train_sum_parts<<<(unsigned) ((nw + 255) / 256), 256>>>(f->part_w, f->zsplit, nw, f->g + OFF_W + (size_t) (l - 1) * nw);
    conv_launch(f->dz[cur], f->dz[cur ^ 1], LP, W2, d, B, f->wtbf + (size_t) (l - 1) * KT * CH * CH, nullptr, f->err, f->act[l - 1]);
    cur ^= 1;
  }
  train_bias_grad<<<NB_BIAS, CH>>>(f->dz[cur], (long long) B * LP, f->part_b);
  train_sum_parts<<<1, CH>>>(f->part_b, NB_BIAS, CH, f->g + OFF_B);
  train_wgrad0<<<NB_W0, CH>>>(f->dz[cur], f->win, B, LP, W2, f->part_w0);
  train_sum_parts<<<(KT * 4 * CH + 255) / 256, 256>>>(f->part_w0, NB_W0, (long long) KT * 4 * CH, f->g + OFF_W0);
  if (lr > 0.f) {
    f->t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = (float) (1.0 - std::pow((double) b1, (double) f->t)), bc2 = (float) (1.0 - std::pow((double) b2, (double) f->t));
    train_adamw<<<512, 256>>>(f->p, f->g, f->m1, f->m2, (long long) NPARAM, lr, b1, b2, 1e-8f, weight_decay, bc1, bc2);
    train_pack<<<512, 256>>>(f->p + OFF_W, f->wbf, f->wtbf);
  }
  FCUDA(cudaGetLastError());
  FCUDA(cudaEventRecord(e1));
  float hl = 0.f; int herr = 0;
  FCUDA(cudaMemcpy(&hl, f->loss, sizeof(float), cudaMemcpyDeviceToHost));
  FCUDA(cudaMemcpy(&herr, f->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) FERR(CMGB_ENODEV, "filter trainer: a bounded tensor-core wait ran out");
  float ms = 0.f;
  FCUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  if (ret_loss) *ret_loss = hl;
  if (ret_ms) *ret_ms = ms;
  return CMGB_OK;
#endif
}

extern "C" int cmgb_filter_trainer_step(cmgb_filter_trainer *f, const uint8_t *windows, const float *labels, float pos_weight,
                                        float lr, float weight_decay, float *ret_loss, float *ret_ms, char *errbuf)
{
  if (!f) FERR(CMGB_EINVAL, "filter trainer: invalid arguments");
  std::vector<float> pw((size_t) f->H, pos_weight);
  return cmgb_filter_trainer_step_heads(f, windows, labels, pw.data(), lr, weight_decay, ret_loss, ret_ms, errbuf);
}

// Copies out the fp32 master weights (set's layout) and, when gw0 != NULL, the
// last step's gradients in the same layout (gw0, gw, gb, gwout).
extern "C" int cmgb_filter_trainer_get(cmgb_filter_trainer *f, float *w0, float *w, float *bias, float *wout,
                                       float *gw0, float *gw, float *gb, float *gwout, char *errbuf)
{
#ifdef CMGB_HOST_EMULATION
  (void) f; (void) w0; (void) w; (void) bias; (void) wout; (void) gw0; (void) gw; (void) gb; (void) gwout;
  FERR(CMGB_ENODEV, "filter trainer: not available in the host emulation");
#else
  if (!f) FERR(CMGB_EINVAL, "filter trainer: invalid arguments");
  const float *src[2] = {f->p, f->g};
  float *dst[2][4] = {{w0, w, bias, wout}, {gw0, gw, gb, gwout}};
  const size_t off[5] = {OFF_W0, OFF_W, OFF_B, OFF_WOUT, f->np};
  for (int k = 0; k < 2; k++)
    for (int j = 0; j < 4; j++)
      if (dst[k][j]) FCUDA(cudaMemcpy(dst[k][j], src[k] + off[j], sizeof(float) * (off[j + 1] - off[j]), cudaMemcpyDeviceToHost));
  return CMGB_OK;
#endif
}
