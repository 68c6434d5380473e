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
// channels, K = 9 taps x 128 input channels) on the tensor cores with
// mma.sync m16n8k16 BF16 -> FP32: a CTA computes a 128 x 128 output tile; its
// input rows for all nine taps (128 + 8 d rows) are staged once in shared
// memory, the tap's weights per tap.
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
constexpr int SROW = CH + 8; // padded shared-memory row (bf16 elements): conflict-free fragment loads
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

__device__ __forceinline__ void mma_bf16(float *c, const unsigned *a, const unsigned *bq)
{
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(bq[0]), "r"(bq[1]));
}

// Layers 1-5: out[w][i][co] = relu(b[co] + sum_t sum_ci in[w][i + (t-4) d][ci] * wt[t][co][ci]).
// Grid: (LP / 128 tiles, nwin); 256 threads = 8 warps, warp (wm, wn) owns
// rows 32 wm .. +32 and columns 64 wn .. +64 of the tile.
__global__ void __launch_bounds__(256) filter_conv(const unsigned short *in, unsigned short *out, int LP, int W2, int dil,
                                                   const unsigned short *wt, const float *bias)
{
  extern __shared__ __align__(16) unsigned short fsm[];
  const int rows = TILE + 8 * dil;             // staged input rows: tile plus the taps' reach
  unsigned short *sA = fsm;                    // [rows][SROW]
  unsigned short *sB = fsm + (size_t) rows * SROW;   // [128 co][SROW]
  const int tile = blockIdx.x, win = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;
  const int g = lane >> 2, tg = lane & 3;
  const int p0 = tile * TILE - 4 * dil;        // window position of staged row 0
  const unsigned short *inw = in + (size_t) win * LP * CH;
  // stage the input rows (16-byte chunks); rows outside [0, LP) are zero
  for (int x = tid; x < rows * (CH / 8); x += blockDim.x) {
    const int r = x / (CH / 8), c8 = x - r * (CH / 8);
    const int p = p0 + r;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (p >= 0 && p < LP) v = *reinterpret_cast<const uint4 *>(inw + (size_t) p * CH + c8 * 8);
    *reinterpret_cast<uint4 *>(sA + (size_t) r * SROW + c8 * 8) = v;
  }
  float acc[2][8][4];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[a][n][q] = 0.f;

  for (int t = 0; t < KT; t++) {
    __syncthreads();   // previous tap's B fully consumed (and, at t = 0, A staged)
    const unsigned short *wtt = wt + (size_t) t * CH * CH;
    for (int x = tid; x < CH * (CH / 8); x += blockDim.x) {
      const int r = x / (CH / 8), c8 = x - r * (CH / 8);
      *reinterpret_cast<uint4 *>(sB + (size_t) r * SROW + c8 * 8) = *reinterpret_cast<const uint4 *>(wtt + (size_t) r * CH + c8 * 8);
    }
    __syncthreads();
    const int rbase = t * dil;                 // staged row of tile row 0 for this tap
#pragma unroll 2
    for (int k0 = 0; k0 < CH; k0 += 16) {
      unsigned af[2][4];
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const int r = rbase + 32 * wm + 16 * a + g;
        const unsigned short *p = sA + (size_t) r * SROW + k0 + 2 * tg;
        af[a][0] = *reinterpret_cast<const unsigned *>(p);
        af[a][1] = *reinterpret_cast<const unsigned *>(p + 8 * SROW);
        af[a][2] = *reinterpret_cast<const unsigned *>(p + 8);
        af[a][3] = *reinterpret_cast<const unsigned *>(p + 8 * SROW + 8);
      }
#pragma unroll
      for (int n = 0; n < 8; n++) {
        const unsigned short *p = sB + (size_t) (64 * wn + 8 * n + g) * SROW + k0 + 2 * tg;
        unsigned bq[2];
        bq[0] = *reinterpret_cast<const unsigned *>(p);
        bq[1] = *reinterpret_cast<const unsigned *>(p + 8);
        mma_bf16(acc[0][n], af[0], bq);
        mma_bf16(acc[1][n], af[1], bq);
      }
    }
  }
  // epilogue: bias, ReLU, BF16; rows at or beyond the window length are zero
  unsigned short *outw = out + (size_t) win * LP * CH;
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const int col = 64 * wn + 8 * n + 2 * tg;
      const float b0 = bias[col], b1 = bias[col + 1];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int row = tile * TILE + 32 * wm + 16 * a + g + 8 * h;
        float v0 = acc[a][n][2 * h] + b0, v1 = acc[a][n][2 * h + 1] + b1;
        v0 = v0 > 0.f ? v0 : 0.f; v1 = v1 > 0.f ? v1 : 0.f;
        if (row >= W2) v0 = v1 = 0.f;
        const unsigned pk = (unsigned) f2bf(v0) | ((unsigned) f2bf(v1) << 16);
        *reinterpret_cast<unsigned *>(outw + (size_t) row * CH + col) = pk;
      }
    }
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
  int maxsm = (TILE + 8 * DIL[NL - 1]) * SROW * 2 + CH * SROW * 2;
  FCUDA(cudaFuncSetAttribute(filter_conv, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm));
  *ret = f.release();
  return CMGB_OK;
#endif
}

extern "C" void cmgb_filter_destroy(cmgb_filter *f)
{
  if (!f) return;
#ifndef CMGB_HOST_EMULATION
  cudaFree(f->d_w0); cudaFree(f->d_w); cudaFree(f->d_b); cudaFree(f->d_out);
  cudaFree(f->d_act[0]); cudaFree(f->d_act[1]); cudaFree(f->d_logit);
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
    const size_t sm = (size_t) (TILE + 8 * d) * SROW * 2 + (size_t) CH * SROW * 2;
    filter_conv<<<dim3(f->LP / TILE, nwin), 256, sm>>>(f->d_act[cur], f->d_act[cur ^ 1], f->LP, (int) (2 * W), d,
                                                       f->d_w + (size_t) (l - 1) * KT * CH * CH, f->d_b + l * CH);
    FCUDA(cudaGetLastError());
    cur ^= 1;
  }
  filter_readout<<<nwin, CH>>>(f->d_act[cur], f->LP, (int) (2 * W), f->d_out, f->d_logit);
  FCUDA(cudaGetLastError());
  FCUDA(cudaEventRecord(e1));
  FCUDA(cudaMemcpy(ret_logits, f->d_logit, sizeof(float) * nwin, cudaMemcpyDeviceToHost));
  float ms = 0.f;
  FCUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  if (ret_nwin) *ret_nwin = nwin;
  if (ret_ms) *ret_ms = ms;
  return CMGB_OK;
#endif
}
