// surrogate.cu -- training data, training and inference of the pair-energy surrogate.
//
// No counterpart in the reference: this is the learned first stage of the
// delayed-acceptance move test (see surrogate.cuh).  Everything runs on the GPU:
//   * samples: every ordered SC-SC pair of a configuration with FP32 segment distance
//     below rcutS gives (features, exact FP64 pair energy - WCA32) -- the exact energy is
//     the parity-tested PairE of pair_energy.cuh;
//   * training: mini-batch Adam on the MSE, forward and backward on the tensor cores
//     (mma.sync m16n8k16, BF16 operands, FP32 accumulation), FP32 master weights,
//     per-CTA gradient partials summed in a fixed order (bit-reproducible);
//   * inference: the same warp-level forward (mlpForward16) the move kernel uses.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include "../../include/sc_gb300.h"
#include "kernels.h"
#include "pair_energy.cuh"
#include "philox.cuh"
#include "sc_context.h"
#include "surrogate.cuh"

namespace scg {
namespace {

constexpr int kTrainThreads = 128;       // 4 warps, 16 rows each
constexpr int kChunkRows = 64;
constexpr int kLd = 72;                  // padded BF16 row stride of the activation tiles (144 B)
constexpr int kLdX = 24;                 // padded BF16 row stride of the input tile (48 B)
constexpr int kPartStride = kParamsPad + 4;   // per-CTA gradient partial + loss
constexpr int kSampleTile = 256;

struct TrainShared {
    __nv_bfloat16 x0[kChunkRows][kLdX];
    __nv_bfloat16 h1[kChunkRows][kLd];
    __nv_bfloat16 h2[kChunkRows][kLd];
    __nv_bfloat16 h3[kChunkRows][kLd];
    __nv_bfloat16 d1[kChunkRows][kLd];
    __nv_bfloat16 d2[kChunkRows][kLd];
    __nv_bfloat16 d3[kChunkRows][kLd];
    float dy[kChunkRows];
};

__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], const void* p) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// Stores a C-layout tile (8 n-tiles of 16 x 8) as BF16 rows r0..r0+15 of T.
__device__ __forceinline__ void storeC(__nv_bfloat16 (*T)[kLd], int r0, const float (&c)[8][4], int lane) {
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        *reinterpret_cast<uint32_t*>(&T[r0 + g][nt * 8 + 2 * q]) = packBf16(c[nt][0], c[nt][1]);
        *reinterpret_cast<uint32_t*>(&T[r0 + g + 8][nt * 8 + 2 * q]) = packBf16(c[nt][2], c[nt][3]);
    }
}

// Backward of a hidden layer: dh = dz W^T with W^T given as fragments T[kt][nt].
__device__ __forceinline__ void backLayer(const uint2 (*T)[8][32], const uint32_t (&dz)[4][4], float (&dh)[8][4],
                                          int lane) {
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) mma16816(c, dz[kt], T[kt][nt][lane], c);
#pragma unroll
        for (int e = 0; e < 4; ++e) dh[nt][e] = c[e];
    }
}

// Weight gradient tiles: acc[mt][j] += A^T B over the 64 rows of the chunk, A = S rows
// (columns 16mt.. of a [64][ld] BF16 tile), B = D rows (columns 8(n0+j)..).
template <int MT, int LDA>
__device__ __forceinline__ void gradGemm(const __nv_bfloat16 (*S)[LDA], const __nv_bfloat16 (*D)[kLd], int n0,
                                         float (&acc)[MT][2][4], int lane) {
    const int j = lane >> 3, r = lane & 7;
#pragma unroll
    for (int ks = 0; ks < kChunkRows / 16; ++ks) {
        uint32_t b[4];
        ldsm4t(b, &D[ks * 16 + (j & 1) * 8 + r][(n0 + (j >> 1)) * 8]);
        uint2 b0 = make_uint2(b[0], b[1]), b1 = make_uint2(b[2], b[3]);
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
            uint32_t a[4];
            ldsm4t(a, &S[ks * 16 + (j >> 1) * 8 + r][mt * 16 + (j & 1) * 8]);
            mma16816(acc[mt][0], a, b0, acc[mt][0]);
            mma16816(acc[mt][1], a, b1, acc[mt][1]);
        }
    }
}

// One training pass over rowsPerCta rows per CTA: forward, MSE gradient, backward, and
// the CTA's gradient partial (+ its squared-error sum) into part[blockIdx.x].
// mode 0: rows drawn uniformly (Philox keyed by seed, step, CTA, row); mode 1: rows in
// order, rows >= n weigh 0.
__global__ void __launch_bounds__(kTrainThreads) kMlpTrain(const MlpPacked* __restrict__ P,
                                                           const float* __restrict__ feats,
                                                           const float* __restrict__ target, long n, int chunks,
                                                           int mode, uint64_t seed, long step, float invBatch,
                                                           float* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char trainSmem[];
    TrainShared& sh = *reinterpret_cast<TrainShared*>(trainSmem);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, q = lane & 3;
    float accW2[4][2][4], accW3[4][2][4], accW1[1][2][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int e = 0; e < 4; ++e) { accW2[a][b][e] = 0.0f; accW3[a][b][e] = 0.0f; }
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int e = 0; e < 4; ++e) accW1[0][b][e] = 0.0f;
    float accS = 0.0f, accS2 = 0.0f;    // thread-owned scalars: dW4 / db2 / db3 / db4 sums
    float lossSum = 0.0f;
    const int r0 = warp * 16;

    for (int ch = 0; ch < chunks; ++ch) {
        // rows of this warp: lanes 0..15 load one row each
        float tgt = 0.0f, wgt = 0.0f;
        if (lane < 16) {
            long idx;
            bool valid = true;
            if (mode == 0) {
                Stream r(seed, (uint32_t)step, (uint32_t)(blockIdx.x * chunks + ch), (uint32_t)(r0 + lane));
                idx = (long)(r.next() * (double)n);
                if (idx >= n) idx = n - 1;
            } else {
                idx = ((long)blockIdx.x * chunks + ch) * kChunkRows + r0 + lane;
                valid = idx < n;
            }
            float f[kFeat];
            if (valid) {
                const float4* src = reinterpret_cast<const float4*>(feats + idx * kFeat);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    float4 v = src[k];
                    f[4 * k] = v.x; f[4 * k + 1] = v.y; f[4 * k + 2] = v.z; f[4 * k + 3] = v.w;
                }
                tgt = target[idx];
                wgt = 1.0f;
            } else {
#pragma unroll
                for (int k = 0; k < kFeat; ++k) f[k] = 0.0f;
            }
#pragma unroll
            for (int k = 0; k < kFeat; k += 2)
                *reinterpret_cast<uint32_t*>(&sh.x0[r0 + lane][k]) = packBf16(f[k], f[k + 1]);
        }
        __syncwarp();
        // ---- forward
        uint32_t a0[4];
        a0[0] = *reinterpret_cast<const uint32_t*>(&sh.x0[r0 + g][2 * q]);
        a0[1] = *reinterpret_cast<const uint32_t*>(&sh.x0[r0 + g + 8][2 * q]);
        a0[2] = *reinterpret_cast<const uint32_t*>(&sh.x0[r0 + g][2 * q + 8]);
        a0[3] = *reinterpret_cast<const uint32_t*>(&sh.x0[r0 + g + 8][2 * q + 8]);
        float z1[8][4], z2[8][4], z3[8][4], hc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma16816(c, a0, P->f1[nt][lane], c);
#pragma unroll
            for (int e = 0; e < 4; ++e) { z1[nt][e] = c[e]; hc[nt][e] = silu(c[e]); }
        }
        storeC(sh.h1, r0, hc, lane);
        uint32_t h[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) cToA(hc[2 * kt], hc[2 * kt + 1], h[kt]);
        hiddenLayer(P->f2, P->b2, h, z2, lane);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) hc[nt][e] = silu(z2[nt][e]);
        storeC(sh.h2, r0, hc, lane);
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) cToA(hc[2 * kt], hc[2 * kt + 1], h[kt]);
        hiddenLayer(P->f3, P->b3, h, z3, lane);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) hc[nt][e] = silu(z3[nt][e]);
        storeC(sh.h3, r0, hc, lane);
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) cToA(hc[2 * kt], hc[2 * kt + 1], h[kt]);
        float y[4] = {P->b4, 0.0f, P->b4, 0.0f};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) mma16816(y, h[kt], P->f4[kt][lane], y);
        // ---- loss gradient: rows g and g+8 live in lane 4g (q == 0)
        float t0 = __shfl_sync(0xffffffffu, tgt, g), t1 = __shfl_sync(0xffffffffu, tgt, g + 8);
        float w0 = __shfl_sync(0xffffffffu, wgt, g), w1 = __shfl_sync(0xffffffffu, wgt, g + 8);
        float y0 = __shfl_sync(0xffffffffu, y[0], lane & ~3), y1 = __shfl_sync(0xffffffffu, y[2], lane & ~3);
        float e0 = y0 - t0, e1 = y1 - t1;
        float dy0 = w0 * 2.0f * e0 * invBatch, dy1 = w1 * 2.0f * e1 * invBatch;
        if (q == 0) {
            lossSum += w0 * e0 * e0 + w1 * e1 * e1;
            sh.dy[r0 + g] = dy0;
            sh.dy[r0 + g + 8] = dy1;
        }
        // ---- backward: dz3 = dy w4 * silu'(z3)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                int col = nt * 8 + 2 * q + (e & 1);
                float w4 = bf16Round(P->w4[col]);
                hc[nt][e] = (e < 2 ? dy0 : dy1) * w4 * siluGrad(z3[nt][e]);
            }
        storeC(sh.d3, r0, hc, lane);
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) cToA(hc[2 * kt], hc[2 * kt + 1], h[kt]);
        backLayer(P->t3, h, hc, lane);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) hc[nt][e] *= siluGrad(z2[nt][e]);
        storeC(sh.d2, r0, hc, lane);
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) cToA(hc[2 * kt], hc[2 * kt + 1], h[kt]);
        backLayer(P->t2, h, hc, lane);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) hc[nt][e] *= siluGrad(z1[nt][e]);
        storeC(sh.d1, r0, hc, lane);
        __syncthreads();
        // ---- weight gradients over the chunk's 64 rows; warp w owns output n-tiles 2w, 2w+1
        gradGemm<4, kLd>(sh.h1, sh.d2, 2 * warp, accW2, lane);
        gradGemm<4, kLd>(sh.h2, sh.d3, 2 * warp, accW3, lane);
        gradGemm<1, kLdX>(sh.x0, sh.d1, 2 * warp, accW1, lane);
        // thread k < 64: dW4[k] and db3[k]; thread 64 + k: db2[k]; (db4 from thread 0's second sum)
        if (tid < 64) {
            float s1 = 0.0f, s2 = 0.0f;
            for (int r = 0; r < kChunkRows; ++r) {
                s1 += __bfloat162float(sh.h3[r][tid]) * sh.dy[r];
                s2 += __bfloat162float(sh.d3[r][tid]);
            }
            accS += s1;
            accS2 += s2;
        } else {
            float s1 = 0.0f, s2 = 0.0f;
            for (int r = 0; r < kChunkRows; ++r) s1 += __bfloat162float(sh.d2[r][tid - 64]);
            if (tid == 64)
                for (int r = 0; r < kChunkRows; ++r) s2 += sh.dy[r];
            accS += s1;
            accS2 += s2;
        }
        __syncthreads();
    }
    // ---- partials
    float* out = part + (size_t)blockIdx.x * kPartStride;
#pragma unroll
    for (int mt = 0; mt < 4; ++mt)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                int row = mt * 16 + g + 8 * (e >> 1);
                int col = (2 * warp + j) * 8 + 2 * q + (e & 1);
                out[kOffW2 + row * kHidden + col] = accW2[mt][j][e];
                out[kOffW3 + row * kHidden + col] = accW3[mt][j][e];
            }
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int row = g + 8 * (e >> 1);
            int col = (2 * warp + j) * 8 + 2 * q + (e & 1);
            out[kOffW1 + row * kHidden + col] = accW1[0][j][e];
        }
    if (tid < 64) {
        out[kOffW4 + tid] = accS;
        out[kOffB3 + tid] = accS2;
    } else {
        out[kOffB2 + tid - 64] = accS;
        if (tid == 64) out[kOffB4] = accS2;
    }
    // loss: warp sums, then warp 0 in a fixed order
    for (int o = 16; o > 0; o >>= 1) lossSum += __shfl_xor_sync(0xffffffffu, lossSum, o);
    __shared__ float lossW[4];
    if (lane == 0) lossW[warp] = lossSum;
    __syncthreads();
    if (tid == 0) out[kParamsPad] = lossW[0] + lossW[1] + lossW[2] + lossW[3];
}

// grad = sum of the CTA partials in CTA order; optionally one Adam step on the masters.
__global__ void kGradAdam(const float* __restrict__ part, int nParts, float* __restrict__ grad, float* theta,
                          float* mom, float* vel, int adam, float lr, float beta1, float beta2, float eps,
                          double* lossOut) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < kParams) {
        float s = 0.0f;
        for (int b = 0; b < nParts; ++b) s += part[(size_t)b * kPartStride + p];
        grad[p] = s;
        if (adam) {
            float m = beta1 * mom[p] + (1.0f - beta1) * s;
            float v = beta2 * vel[p] + (1.0f - beta2) * s * s;
            mom[p] = m;
            vel[p] = v;
            theta[p] -= lr * m / (sqrtf(v) + eps);
        }
    } else if (p == kParams && lossOut) {
        double s = 0.0;
        for (int b = 0; b < nParts; ++b) s += (double)part[(size_t)b * kPartStride + kParamsPad];
        *lossOut = s;
    }
}

__device__ __forceinline__ float wAt(const float* th, int off, int K, int N, int k, int n) {
    return (k < K && n < N) ? th[off + k * N + n] : 0.0f;
}

// Packs the FP32 masters into the BF16 fragment blocks of MlpPacked.
__global__ void kMlpPack(const float* __restrict__ th, MlpPacked* P, float rcutS) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    // blocks: f1 8, f2 32, f3 32, f4 4, t2 32, t3 32
    const int nb = 8 + 32 + 32 + 4 + 32 + 32;
    if (i < nb * 32) {
        int blk = i >> 5, lane = i & 31;
        int g = lane >> 2, q = lane & 3;
        int off, K, N, kt, nt, trans = 0;
        uint2* dst;
        if (blk < 8) { off = kOffW1; K = kFeat; N = kHidden; kt = 0; nt = blk; dst = &P->f1[nt][lane]; }
        else if (blk < 40) { int b = blk - 8; kt = b >> 3; nt = b & 7; off = kOffW2; K = N = kHidden; dst = &P->f2[kt][nt][lane]; }
        else if (blk < 72) { int b = blk - 40; kt = b >> 3; nt = b & 7; off = kOffW3; K = N = kHidden; dst = &P->f3[kt][nt][lane]; }
        else if (blk < 76) { kt = blk - 72; nt = 0; off = kOffW4; K = kHidden; N = 1; dst = &P->f4[kt][lane]; }
        else if (blk < 108) { int b = blk - 76; kt = b >> 3; nt = b & 7; off = kOffW2; K = N = kHidden; trans = 1; dst = &P->t2[kt][nt][lane]; }
        else { int b = blk - 108; kt = b >> 3; nt = b & 7; off = kOffW3; K = N = kHidden; trans = 1; dst = &P->t3[kt][nt][lane]; }
        int k0 = kt * 16 + 2 * q, n = nt * 8 + g;
        float v[4];
        for (int e = 0; e < 4; ++e) {
            int k = k0 + (e & 1) + 8 * (e >> 1);
            v[e] = trans ? wAt(th, off, K, N, n, k) : wAt(th, off, K, N, k, n);
        }
        *dst = make_uint2(packBf16(v[0], v[1]), packBf16(v[2], v[3]));
    }
    if (i < kHidden) {
        P->b2[i] = th[kOffB2 + i];
        P->b3[i] = th[kOffB3 + i];
        P->w4[i] = th[kOffW4 + i];
    }
    if (i == 0) {
        P->b4 = th[kOffB4];
        P->rcutS = rcutS;
    }
}

// Inference over n rows of features (warp per 16 rows) -- the move kernel's forward.
__global__ void kMlpPredict(const MlpPacked* __restrict__ P, const float* __restrict__ feats, int n,
                            float* __restrict__ out) {
    __shared__ float X[4][16][kFeat];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = (blockIdx.x * 4 + warp) * 16;
    if (row0 >= n) return;
    if (lane < 16) {
        int r = row0 + lane;
        for (int k = 0; k < kFeat; ++k) X[warp][lane][k] = r < n ? feats[(size_t)r * kFeat + k] : 0.0f;
    }
    __syncwarp();
    float y0, y1;
    mlpForward16(P, X[warp], y0, y1);
    if ((lane & 3) == 0) {
        int g = lane >> 2;
        if (row0 + g < n) out[row0 + g] = y0;
        if (row0 + g + 8 < n) out[row0 + g + 8] = y1;
    }
}

// ---- training samples from a configuration --------------------------------------------

struct SampleArgs {
    DevState s;
    DevTables t;
    const float4* posF;     // wrapped FP32 box fractions, w = compact type
    const float4* dirF;     // FP32 axis
    const float4* patF;     // FP32 first patch direction
    float rcutS;
    float wcaMax;           // pairs whose WCA32 exceeds this are left out (cancellation)
};

__global__ void kPrepF32(DevState s, float4* posF, float4* dirF, float4* patF) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    double4_32a p = s.pos[i], d = s.dir[i];
    posF[i] = make_float4(frac32(p.x), frac32(p.y), frac32(p.z), (float)p.w);
    dirF[i] = make_float4((float)d.x, (float)d.y, (float)d.z, 0.0f);
    const PatchSet& ps = s.patch[i];
    patF[i] = make_float4((float)ps.pd[0][0], (float)ps.pd[0][1], (float)ps.pd[0][2], 0.0f);
}


// Features, WCA32 and eligibility of given ordered pairs (i, j): what the move kernel
// computes for particle i moved against neighbour j.
__global__ void kPairFeatures(DevState s, DevTables t, int npairs, const int* I, const int* J, float rcutS,
                              float* feats, float* wca, int* elig) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npairs) return;
    int i = I[k], j = J[k];
    double4_32a p1 = s.pos[i], p2 = s.pos[j], d1 = s.dir[i], d2 = s.dir[j];
    int ti = (int)p1.w, tj = (int)p2.w;
    const PairParam& pp = t.params[ti * t.ntypes + tj];
    float3 ci = make_float3(frac32(p1.x), frac32(p1.y), frac32(p1.z));
    float4 cj = make_float4(frac32(p2.x), frac32(p2.y), frac32(p2.z), 0.0f);
    float3 r = pairVecF(ci, cj, (float)s.box[0], (float)s.box[1], (float)s.box[2]);
    const PatchSet& q1 = s.patch[i];
    const PatchSet& q2 = s.patch[j];
    float f[kFeat];
    float dd = pairFeatures(r, make_float3((float)d1.x, (float)d1.y, (float)d1.z),
                            make_float3((float)q1.pd[0][0], (float)q1.pd[0][1], (float)q1.pd[0][2]),
                            (float)pp.half_len[0], typeCode(ti, t.ntypes),
                            make_float3((float)d2.x, (float)d2.y, (float)d2.z),
                            make_float3((float)q2.pd[0][0], (float)q2.pd[0][1], (float)q2.pd[0][2]),
                            (float)pp.half_len[1], typeCode(tj, t.ntypes), f);
    for (int q = 0; q < kFeat; ++q) feats[(size_t)k * kFeat + q] = f[q];
    DevCtx c;
    c.params = t.params; c.mols = t.mols; c.ntypes = t.ntypes; c.n = s.n; c.sqmaxcut = t.sqmaxcut;
    Con con = makeCon(c, i, s.mol[i]);
    bool bonded = (j == con.idx[0] || j == con.idx[1] || j == con.idx[2] || j == con.idx[3]);
    bool ok = pp.screen == 1 && !bonded && dd < rcutS * rcutS;
    elig[k] = ok ? 1 : 0;
    wca[k] = ok ? wca32(dd, (float)pp.sigma, (float)pp.epsilon, (float)pp.rcutwcaSq) : 0.0f;
}

// Pass 1 (write == false): count[i] = samples of particle i.  Pass 2: writes them at
// offset[i] (features, target = exact pair energy - WCA32).  Thread per particle i,
// every j != i in tiles of kSampleTile.
template <bool write>
__global__ void __launch_bounds__(kSampleTile) kSamplePairs(SampleArgs A, int* count, const long* offset,
                                                            float* feats, float* target, long cap) {
    __shared__ float4 tp[kSampleTile], td[kSampleTile];
    const int n = A.s.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double bxd = A.s.box[0], byd = A.s.box[1], bzd = A.s.box[2];
    const float bx = (float)bxd, by = (float)byd, bz = (float)bzd;
    float4 pi = i < n ? A.posF[i] : make_float4(0, 0, 0, 0);
    float4 di = i < n ? A.dirF[i] : make_float4(0, 0, 0, 0);
    const int ti = (int)pi.w;
    const float3 ci = make_float3(pi.x, pi.y, pi.z);
    const float3 ai = make_float3(di.x, di.y, di.z);
    DevCtx c;
    c.params = A.t.params; c.mols = A.t.mols; c.ntypes = A.t.ntypes; c.n = n; c.sqmaxcut = A.t.sqmaxcut;
    Con con{};
    if (i < n) con = makeCon(c, i, A.s.mol[i]);
    int cnt = 0;
    long out = write && i < n ? offset[i] : 0;
    const float rc2 = A.rcutS * A.rcutS;
    for (int base = 0; base < n; base += kSampleTile) {
        __syncthreads();
        if (base + threadIdx.x < n) {
            tp[threadIdx.x] = A.posF[base + threadIdx.x];
            td[threadIdx.x] = A.dirF[base + threadIdx.x];
        }
        __syncthreads();
        if (i >= n) continue;
        const int m = min(kSampleTile, n - base);
        for (int k = 0; k < m; ++k) {
            const int j = base + k;
            if (j == i) continue;
            const float4 pj = tp[k];
            const int tj = (int)pj.w;
            const PairParam& pp = c.params[ti * c.ntypes + tj];
            if (pp.screen != 1) continue;
            float3 r = pairVecF(ci, pj, bx, by, bz);
            float reach = A.rcutS + (float)pp.half_len[0] + (float)pp.half_len[1];
            if (dotf(r, r) > reach * reach) continue;
            if (j == con.idx[0] || j == con.idx[1] || j == con.idx[2] || j == con.idx[3]) continue;
            float s, t;
            float3 w;
            float d2 = segClosestF(r, ai, make_float3(td[k].x, td[k].y, td[k].z), (float)pp.half_len[0],
                                   (float)pp.half_len[1], s, t, w);
            if (!(d2 < rc2)) continue;
            float wca = wca32(d2, (float)pp.sigma, (float)pp.epsilon, (float)pp.rcutwcaSq);
            if (wca > A.wcaMax) continue;
            if (write) {
                if (out < cap) {
                    float4 pa = A.patF[i], pb = A.patF[j];
                    float f[kFeat];
                    pairFeatures(r, ai, make_float3(pa.x, pa.y, pa.z), (float)pp.half_len[0], typeCode(ti, c.ntypes),
                                 make_float3(td[k].x, td[k].y, td[k].z), make_float3(pb.x, pb.y, pb.z),
                                 (float)pp.half_len[1], typeCode(tj, c.ntypes), f);
                    float4* dst = reinterpret_cast<float4*>(feats + out * kFeat);
                    for (int q = 0; q < 4; ++q) dst[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
                    PView va, vb;
                    double4_32a p1 = A.s.pos[i], p2 = A.s.pos[j], d1 = A.s.dir[i], d2v = A.s.dir[j];
                    va.pos = mk(p1.x, p1.y, p1.z); va.dir = mk(d1.x, d1.y, d1.z); va.patch = &A.s.patch[i];
                    va.type = ti; va.index = i; va.molType = 0;
                    vb.pos = mk(p2.x, p2.y, p2.z); vb.dir = mk(d2v.x, d2v.y, d2v.z); vb.patch = &A.s.patch[j];
                    vb.type = tj; vb.index = j; vb.molType = 0;
                    unsigned bits;
                    double dd;
                    double e = pairEnergy(c, va, vb, con, mk(bxd, byd, bzd), &bits, &dd);
                    target[out] = (float)(e - (double)wca);
                }
                ++out;
            }
            ++cnt;
        }
    }
    if (!write && i < n) count[i] = cnt;
}

}  // namespace

// ---- host side ------------------------------------------------------------------------------

struct Surrogate {
    int device = 0;
    cudaStream_t stream = nullptr;
    float* theta = nullptr;    // FP32 masters
    float* mom = nullptr;
    float* vel = nullptr;
    float* grad = nullptr;
    MlpPacked* packed = nullptr;
    float* part = nullptr;
    int partCap = 0;
    double* dLoss = nullptr;
    float* feats = nullptr;    // training set
    float* target = nullptr;
    long cap = 0, count = 0;
    long adamStep = 0;
    float rcutS = 0.0f;
    int ntypes = 0;
    uint64_t seed = 1;
};

static int surFail(cudaError_t e, const char* where) { return cudaFail(e, where); }

static int packWeights(Surrogate* s) {
    kMlpPack<<<(140 * 32 + 255) / 256, 256, 0, s->stream>>>(s->theta, s->packed, s->rcutS);
    cudaError_t r = cudaGetLastError();
    return r == cudaSuccess ? SC_OK : surFail(r, "surrogate pack");
}

// Largest rcut over SC-SC pair classes of the context's types (the surrogate's range).
float surrogateRange(Context* c) {
    double r = 0.0;
    int nt = (int)c->usedTypes.size();
    for (int a = 0; a < nt; ++a)
        for (int b = 0; b < nt; ++b) {
            PairParam pp = c->devParam(c->usedTypes[a], c->usedTypes[b]);
            if (pp.screen == 1) r = std::max(r, pp.rcut);
        }
    return (float)r;
}

static int ensurePart(Surrogate* s, int nParts) {
    if (nParts <= s->partCap) return SC_OK;
    if (s->part) cudaFree(s->part);
    s->part = nullptr;
    cudaError_t r = cudaMalloc(&s->part, (size_t)nParts * kPartStride * sizeof(float));
    if (r != cudaSuccess) return surFail(r, "surrogate partials");
    s->partCap = nParts;
    return SC_OK;
}

static int trainStep(Surrogate* s, const float* feats, const float* target, long n, int nCta, int chunks, int mode,
                     long step, float invBatch, int adam, float lr) {
    int rc = ensurePart(s, nCta);
    if (rc) return rc;
    kMlpTrain<<<nCta, kTrainThreads, sizeof(TrainShared), s->stream>>>(s->packed, feats, target, n, chunks, mode,
                                                                       s->seed, step, invBatch, s->part);
    kGradAdam<<<(kParams + 1 + 255) / 256, 256, 0, s->stream>>>(s->part, nCta, s->grad, s->theta, s->mom, s->vel, adam,
                                                                lr, 0.9f, 0.999f, 1e-8f, s->dLoss);
    cudaError_t r = cudaGetLastError();
    if (r != cudaSuccess) return surFail(r, "surrogate train step");
    if (adam) return packWeights(s);
    return SC_OK;
}

static void initWeights(std::vector<float>& th, uint64_t seed) {
    th.assign(kParamsPad, 0.0f);
    std::mt19937_64 gen(seed);
    auto fill = [&](int off, int fanIn, int count) {
        float b = std::sqrt(6.0f / (float)fanIn) * 0.5f;
        std::uniform_real_distribution<float> u(-b, b);
        for (int k = 0; k < count; ++k) th[off + k] = u(gen);
    };
    fill(kOffW1, 13, 13 * kHidden);          // rows 0..12 (features + bias); rows 13..15 stay 0
    fill(kOffW2, kHidden, kHidden * kHidden);
    fill(kOffW3, kHidden, kHidden * kHidden);
    fill(kOffW4, kHidden, kHidden);
}

const MlpPacked* surrogatePacked(const Surrogate* s) { return s ? s->packed : nullptr; }
int surrogateDevice(const Surrogate* s) { return s->device; }
float surrogateCutoff(const Surrogate* s) { return s->rcutS; }

}  // namespace scg

using namespace scg;

struct sc_surrogate {
    Surrogate impl;
};

extern "C" {

int sc_surrogate_create(sc_context* ctx, unsigned long long seed, long capacity, sc_surrogate** out) {
    if (!ctx || !out || capacity < 0) return fail(SC_ERR_ARG, "sc_surrogate_create: bad arguments");
    Context* c = reinterpret_cast<Context*>(ctx);
    DeviceScope dev(c->device);
    int rc = c->ensureDevice();
    if (rc) return rc;
    sc_surrogate* h = new sc_surrogate();
    Surrogate& s = h->impl;
    s.device = c->device;
    s.seed = seed;
    s.cap = capacity;
    s.rcutS = surrogateRange(c);
    s.ntypes = (int)c->usedTypes.size();
    cudaError_t r = cudaSetDevice(s.device);
    if (r == cudaSuccess) r = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
    if (r == cudaSuccess) r = cudaMalloc(&s.theta, kParamsPad * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&s.mom, kParamsPad * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&s.vel, kParamsPad * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&s.grad, kParamsPad * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&s.packed, sizeof(MlpPacked));
    if (r == cudaSuccess) r = cudaMalloc(&s.dLoss, sizeof(double));
    if (r == cudaSuccess && capacity > 0) r = cudaMalloc(&s.feats, (size_t)capacity * kFeat * sizeof(float));
    if (r == cudaSuccess && capacity > 0) r = cudaMalloc(&s.target, (size_t)capacity * sizeof(float));
    if (r != cudaSuccess) {
        sc_surrogate_destroy(h);
        return surFail(r, "sc_surrogate_create");
    }
    std::vector<float> th;
    initWeights(th, seed);
    cudaMemcpyAsync(s.theta, th.data(), kParamsPad * sizeof(float), cudaMemcpyHostToDevice, s.stream);
    cudaMemsetAsync(s.mom, 0, kParamsPad * sizeof(float), s.stream);
    cudaMemsetAsync(s.vel, 0, kParamsPad * sizeof(float), s.stream);
    cudaFuncSetAttribute(kMlpTrain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainShared));
    if ((rc = packWeights(&s))) { sc_surrogate_destroy(h); return rc; }
    if ((r = cudaStreamSynchronize(s.stream)) != cudaSuccess) { sc_surrogate_destroy(h); return surFail(r, "create"); }
    *out = h;
    return SC_OK;
}

int sc_surrogate_destroy(sc_surrogate* h) {
    if (!h) return SC_OK;
    Surrogate& s = h->impl;
    DeviceScope dev(s.device);
    if (s.stream) cudaStreamSynchronize(s.stream);
    void* ptrs[] = {s.theta, s.mom, s.vel, s.grad, s.packed, s.part, s.dLoss, s.feats, s.target};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s.stream) cudaStreamDestroy(s.stream);
    delete h;
    return SC_OK;
}

int sc_surrogate_get_weights(sc_surrogate* h, float* out) {
    if (!h || !out) return fail(SC_ERR_ARG, "sc_surrogate_get_weights: null argument");
    Surrogate& s = h->impl;
    DeviceScope dev(s.device);
    cudaError_t r = cudaMemcpyAsync(out, s.theta, kParams * sizeof(float), cudaMemcpyDeviceToHost, s.stream);
    if (r == cudaSuccess) r = cudaStreamSynchronize(s.stream);
    return r == cudaSuccess ? SC_OK : surFail(r, "sc_surrogate_get_weights");
}

int sc_surrogate_set_weights(sc_surrogate* h, const float* in) {
    if (!h || !in) return fail(SC_ERR_ARG, "sc_surrogate_set_weights: null argument");
    Surrogate& s = h->impl;
    DeviceScope dev(s.device);
    std::vector<float> th(kParamsPad, 0.0f);
    std::memcpy(th.data(), in, kParams * sizeof(float));
    for (int k = 13 * kHidden; k < kFeat * kHidden; ++k) th[kOffW1 + k] = 0.0f;   // zero inputs 13..15
    cudaError_t r = cudaMemcpyAsync(s.theta, th.data(), kParamsPad * sizeof(float), cudaMemcpyHostToDevice, s.stream);
    if (r != cudaSuccess) return surFail(r, "sc_surrogate_set_weights");
    cudaMemsetAsync(s.mom, 0, kParamsPad * sizeof(float), s.stream);
    cudaMemsetAsync(s.vel, 0, kParamsPad * sizeof(float), s.stream);
    s.adamStep = 0;
    int rc = packWeights(&s);
    if (rc) return rc;
    r = cudaStreamSynchronize(s.stream);
    return r == cudaSuccess ? SC_OK : surFail(r, "sc_surrogate_set_weights");
}

int sc_surrogate_num_samples(const sc_surrogate* h, long* n) {
    if (!h || !n) return fail(SC_ERR_ARG, "sc_surrogate_num_samples: null argument");
    *n = h->impl.count;
    return SC_OK;
}

// Samples of the context's current configuration: into the training set (dst == NULL) or
// into caller-owned device arrays.
static int samplePairs(Surrogate& s, Context* c, float* feats, float* target, long cap, long* produced) {
    int rc = c->ensureDevice();
    if (rc) return rc;
    if (c->hostNewer && (rc = c->uploadState())) return rc;
    const int n = c->d.n;
    cudaStream_t st = s.stream;
    cudaError_t r;
    // the context's stream may still be moving particles
    if ((r = cudaStreamSynchronize(c->stream)) != cudaSuccess) return surFail(r, "sample: context stream");
    float4 *posF = nullptr, *dirF = nullptr, *patF = nullptr;
    int* count = nullptr;
    long* offset = nullptr;
    r = cudaMalloc(&posF, (size_t)n * sizeof(float4) * 3);
    if (r == cudaSuccess) r = cudaMalloc(&count, (size_t)n * sizeof(int));
    if (r == cudaSuccess) r = cudaMalloc(&offset, (size_t)n * sizeof(long));
    if (r != cudaSuccess) {
        cudaFree(posF); cudaFree(count); cudaFree(offset);
        return surFail(r, "sample: allocation");
    }
    dirF = posF + n;
    patF = dirF + n;
    SampleArgs A;
    A.s = c->d;
    A.t = c->tables;
    A.posF = posF; A.dirF = dirF; A.patF = patF;
    A.rcutS = s.rcutS;
    A.wcaMax = 50.0f;
    const int blocks = (n + kSampleTile - 1) / kSampleTile;
    kPrepF32<<<(n + 255) / 256, 256, 0, st>>>(c->d, posF, dirF, patF);
    kSamplePairs<false><<<blocks, kSampleTile, 0, st>>>(A, count, nullptr, nullptr, nullptr, 0);
    std::vector<int> hc(n);
    r = cudaMemcpyAsync(hc.data(), count, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (r == cudaSuccess) r = cudaStreamSynchronize(st);
    std::vector<long> off(n);
    long tot = 0;
    for (int i = 0; i < n; ++i) { off[i] = tot; tot += hc[i]; }
    if (r == cudaSuccess) r = cudaMemcpyAsync(offset, off.data(), (size_t)n * sizeof(long), cudaMemcpyHostToDevice, st);
    if (r == cudaSuccess) {
        kSamplePairs<true><<<blocks, kSampleTile, 0, st>>>(A, count, offset, feats, target, cap);
        r = cudaGetLastError();
    }
    if (r == cudaSuccess) r = cudaStreamSynchronize(st);
    cudaFree(posF); cudaFree(count); cudaFree(offset);
    if (r != cudaSuccess) return surFail(r, "sample pairs");
    *produced = std::min(tot, cap);
    return SC_OK;
}

int sc_surrogate_collect(sc_surrogate* h, sc_context* ctx, long* total) {
    if (!h || !ctx) return fail(SC_ERR_ARG, "sc_surrogate_collect: null argument");
    Surrogate& s = h->impl;
    Context* c = reinterpret_cast<Context*>(ctx);
    if (c->device != s.device) return fail(SC_ERR_ARG, "sc_surrogate_collect: context on another device");
    DeviceScope dev(s.device);
    long got = 0;
    long room = s.cap - s.count;
    if (room > 0) {
        int rc = samplePairs(s, c, s.feats + s.count * kFeat, s.target + s.count, room, &got);
        if (rc) return rc;
        s.count += got;
    }
    if (total) *total = s.count;
    return SC_OK;
}

int sc_surrogate_train(sc_surrogate* h, const sc_train_params* p, double* loss_per_epoch, sc_train_stats* stats) {
    if (!h || !p) return fail(SC_ERR_ARG, "sc_surrogate_train: null argument");
    Surrogate& s = h->impl;
    if (s.count <= 0) return fail(SC_ERR_STATE, "sc_surrogate_train: no samples collected");
    if (p->epochs < 0 || p->batch < kChunkRows || p->batch % kChunkRows || !(p->lr > 0))
        return fail(SC_ERR_ARG, "sc_surrogate_train: epochs >= 0, batch a multiple of 64, lr > 0");
    DeviceScope dev(s.device);
    const int rowsPerCta = p->batch >= 64 * 152 * 2 ? 128 : 64;
    const int nCta = p->batch / rowsPerCta;
    const int chunks = rowsPerCta / kChunkRows;
    const long stepsPerEpoch = std::max(1L, s.count / p->batch);
    const long total = stepsPerEpoch * p->epochs;
    const float invBatch = 1.0f / (float)p->batch;
    const double lrMin = p->lr_final > 0 ? p->lr_final : p->lr * 0.02;
    auto t0 = std::chrono::steady_clock::now();
    double first = -1.0, last = -1.0;
    long k = 0;
    for (int ep = 0; ep < p->epochs; ++ep) {
        double epochLoss = 0.0;
        for (long it = 0; it < stepsPerEpoch; ++it, ++k) {
            // linear warm-up, cosine decay
            double lr = lrMin + 0.5 * (p->lr - lrMin) * (1.0 + std::cos(M_PI * (double)k / (double)total));
            if (k < p->warmup_steps) lr *= (double)(k + 1) / (double)p->warmup_steps;
            ++s.adamStep;
            double bc = std::sqrt(1.0 - std::pow(0.999, (double)s.adamStep)) / (1.0 - std::pow(0.9, (double)s.adamStep));
            int rc = trainStep(&s, s.feats, s.target, s.count, nCta, chunks, 0, (long)(p->seed * 1000003ull) + k, invBatch,
                               1, (float)(lr * bc));
            if (rc) return rc;
            if (it == stepsPerEpoch - 1 || (ep == 0 && it == 0)) {
                double l = 0.0;
                cudaError_t r = cudaMemcpyAsync(&l, s.dLoss, sizeof(double), cudaMemcpyDeviceToHost, s.stream);
                if (r == cudaSuccess) r = cudaStreamSynchronize(s.stream);
                if (r != cudaSuccess) return surFail(r, "sc_surrogate_train");
                l /= (double)p->batch;
                if (first < 0) first = l;
                last = l;
                epochLoss = l;
            }
        }
        if (loss_per_epoch) loss_per_epoch[ep] = epochLoss;
    }
    cudaError_t r = cudaStreamSynchronize(s.stream);
    if (r != cudaSuccess) return surFail(r, "sc_surrogate_train");
    if (stats) {
        stats->steps = k;
        stats->samples = s.count;
        stats->loss_first = first;
        stats->loss_last = last;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return SC_OK;
}

int sc_surrogate_gradient(sc_surrogate* h, int n, const float* feats, const float* targets, float* grad_out,
                          double* loss) {
    if (!h || n <= 0 || !feats || !targets || !grad_out) return fail(SC_ERR_ARG, "sc_surrogate_gradient: bad arguments");
    Surrogate& s = h->impl;
    DeviceScope dev(s.device);
    float *df = nullptr, *dt = nullptr;
    cudaError_t r = cudaMalloc(&df, (size_t)n * kFeat * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&dt, (size_t)n * sizeof(float));
    if (r == cudaSuccess) r = cudaMemcpyAsync(df, feats, (size_t)n * kFeat * sizeof(float), cudaMemcpyHostToDevice, s.stream);
    if (r == cudaSuccess) r = cudaMemcpyAsync(dt, targets, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s.stream);
    int rc = SC_OK;
    if (r == cudaSuccess) {
        int nCta = (n + kChunkRows - 1) / kChunkRows;
        rc = trainStep(&s, df, dt, n, nCta, 1, 1, 0, 1.0f / (float)n, 0, 0.0f);
    }
    double l = 0.0;
    if (r == cudaSuccess && !rc) r = cudaMemcpyAsync(grad_out, s.grad, kParams * sizeof(float), cudaMemcpyDeviceToHost, s.stream);
    if (r == cudaSuccess && !rc) r = cudaMemcpyAsync(&l, s.dLoss, sizeof(double), cudaMemcpyDeviceToHost, s.stream);
    if (r == cudaSuccess) r = cudaStreamSynchronize(s.stream);
    cudaFree(df);
    cudaFree(dt);
    if (rc) return rc;
    if (r != cudaSuccess) return surFail(r, "sc_surrogate_gradient");
    if (loss) *loss = l / (double)n;
    return SC_OK;
}

int sc_surrogate_predict(sc_surrogate* h, int n, const float* feats, float* out) {
    if (!h || n < 0 || (n && (!feats || !out))) return fail(SC_ERR_ARG, "sc_surrogate_predict: bad arguments");
    if (n == 0) return SC_OK;
    Surrogate& s = h->impl;
    DeviceScope dev(s.device);
    float *df = nullptr, *dy = nullptr;
    cudaError_t r = cudaMalloc(&df, (size_t)n * kFeat * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&dy, (size_t)n * sizeof(float));
    if (r == cudaSuccess) r = cudaMemcpyAsync(df, feats, (size_t)n * kFeat * sizeof(float), cudaMemcpyHostToDevice, s.stream);
    if (r == cudaSuccess) {
        kMlpPredict<<<(n + 63) / 64, 128, 0, s.stream>>>(s.packed, df, n, dy);
        r = cudaGetLastError();
    }
    if (r == cudaSuccess) r = cudaMemcpyAsync(out, dy, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s.stream);
    if (r == cudaSuccess) r = cudaStreamSynchronize(s.stream);
    cudaFree(df);
    cudaFree(dy);
    return r == cudaSuccess ? SC_OK : surFail(r, "sc_surrogate_predict");
}

int sc_surrogate_evaluate(sc_surrogate* h, sc_context* ctx, double* rmse, double* mae, double* max_abs, long* npairs) {
    if (!h || !ctx) return fail(SC_ERR_ARG, "sc_surrogate_evaluate: null argument");
    Surrogate& s = h->impl;
    Context* c = reinterpret_cast<Context*>(ctx);
    DeviceScope dev(s.device);
    const long cap = (long)c->d.n * 64 + 1024;
    float *df = nullptr, *dt = nullptr, *dy = nullptr;
    cudaError_t r = cudaMalloc(&df, (size_t)cap * kFeat * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&dt, (size_t)cap * sizeof(float));
    if (r == cudaSuccess) r = cudaMalloc(&dy, (size_t)cap * sizeof(float));
    if (r != cudaSuccess) {
        cudaFree(df); cudaFree(dt); cudaFree(dy);
        return surFail(r, "sc_surrogate_evaluate");
    }
    long got = 0;
    int rc = samplePairs(s, c, df, dt, cap, &got);
    std::vector<float> ht(got), hy(got);
    if (!rc && got > 0) {
        kMlpPredict<<<(int)((got + 63) / 64), 128, 0, s.stream>>>(s.packed, df, (int)got, dy);
        r = cudaGetLastError();
        if (r == cudaSuccess) r = cudaMemcpyAsync(ht.data(), dt, got * sizeof(float), cudaMemcpyDeviceToHost, s.stream);
        if (r == cudaSuccess) r = cudaMemcpyAsync(hy.data(), dy, got * sizeof(float), cudaMemcpyDeviceToHost, s.stream);
        if (r == cudaSuccess) r = cudaStreamSynchronize(s.stream);
    }
    cudaFree(df); cudaFree(dt); cudaFree(dy);
    if (rc) return rc;
    if (r != cudaSuccess) return surFail(r, "sc_surrogate_evaluate");
    double s2 = 0.0, s1 = 0.0, mx = 0.0;
    for (long k = 0; k < got; ++k) {
        double e = (double)hy[k] - (double)ht[k];
        s2 += e * e;
        s1 += std::fabs(e);
        mx = std::max(mx, std::fabs(e));
    }
    if (rmse) *rmse = got ? std::sqrt(s2 / got) : 0.0;
    if (mae) *mae = got ? s1 / got : 0.0;
    if (max_abs) *max_abs = mx;
    if (npairs) *npairs = got;
    return SC_OK;
}

int sc_pair_features(sc_context* ctx, int npairs, const int* I, const int* J, float* feats, float* wca,
                     int* eligible) {
    if (!ctx || npairs < 0 || (npairs && (!I || !J || !feats || !wca || !eligible)))
        return fail(SC_ERR_ARG, "sc_pair_features: bad arguments");
    Context* c = reinterpret_cast<Context*>(ctx);
    DeviceScope dev(c->device);
    int rc = c->ensureDevice();
    if (rc) return rc;
    for (int k = 0; k < npairs; ++k)
        if (I[k] < 0 || I[k] >= c->d.n || J[k] < 0 || J[k] >= c->d.n || I[k] == J[k])
            return fail(SC_ERR_RANGE, "sc_pair_features: particle index out of range");
    if (npairs == 0) return SC_OK;
    if (c->hostNewer && (rc = c->uploadState())) return rc;
    const float rcutS = surrogateRange(c);
    size_t bytes = (size_t)npairs * (2 * sizeof(int) + (kFeat + 1) * sizeof(float) + sizeof(int));
    if ((rc = c->scratch(bytes))) return rc;
    int* dI = static_cast<int*>(c->dScratch);
    int* dJ = dI + npairs;
    float* dF = reinterpret_cast<float*>(dJ + npairs);
    float* dW = dF + (size_t)npairs * kFeat;
    int* dE = reinterpret_cast<int*>(dW + npairs);
    cudaStream_t st = c->stream;
    cudaError_t r = cudaMemcpyAsync(dI, I, npairs * sizeof(int), cudaMemcpyHostToDevice, st);
    if (r == cudaSuccess) r = cudaMemcpyAsync(dJ, J, npairs * sizeof(int), cudaMemcpyHostToDevice, st);
    if (r == cudaSuccess) {
        kPairFeatures<<<(npairs + 127) / 128, 128, 0, st>>>(c->d, c->tables, npairs, dI, dJ, rcutS, dF, dW, dE);
        r = cudaGetLastError();
    }
    if (r == cudaSuccess) r = cudaMemcpyAsync(feats, dF, (size_t)npairs * kFeat * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (r == cudaSuccess) r = cudaMemcpyAsync(wca, dW, npairs * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (r == cudaSuccess) r = cudaMemcpyAsync(eligible, dE, npairs * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (r == cudaSuccess) r = cudaStreamSynchronize(st);
    return r == cudaSuccess ? SC_OK : surFail(r, "sc_pair_features");
}

int sc_set_surrogate(sc_context* ctx, sc_surrogate* h) {
    if (!ctx) return fail(SC_ERR_ARG, "sc_set_surrogate: null context");
    Context* c = reinterpret_cast<Context*>(ctx);
    if (h) {
        DeviceScope dev(c->device);
        int rc = c->ensureDevice();
        if (rc) return rc;
        if (h->impl.device != c->device) return fail(SC_ERR_ARG, "sc_set_surrogate: surrogate on another device");
        if ((int)c->usedTypes.size() != h->impl.ntypes)
            return fail(SC_ERR_ARG, "sc_set_surrogate: surrogate built for another set of types");
    }
    c->surrogate = h ? &h->impl : nullptr;
    return SC_OK;
}

}  // extern "C"
