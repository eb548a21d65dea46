// surrogate.cuh -- learned pair-energy surrogate: pair features and the BF16 tensor-core MLP.
//
// There is no counterpart in the reference (robertvacha/SC computes every pair energy
// exactly).  The surrogate is the first stage of a two-stage (delayed-acceptance)
// Metropolis test: a move is first accepted with min(1, exp(-dEs/T)), dEs the
// surrogate's energy change, and only then with min(1, exp(-(dE - dEs)/T)), dE the
// exact FP64 change.  For a symmetric proposal the product of the two ratios obeys
// detailed balance with respect to the exact Boltzmann weight whenever
// dEs(x->y) = -dEs(y->x), which holds because dEs is a sum of one deterministic pair
// function over the moved particle's pairs, new minus old.
//
// Surrogate pair energy of an SC-SC pair (PairParam::screen == 1):
//     s(i, j) = WCA32(d) + MLP(features(i, j))        if d < rcutS,   else 0,
// d the FP32 closest distance of the two segments, WCA32 the reference's truncated
// WCA (paire.h:385-393) in FP32 on d, MLP a 16 -> 64 -> 64 -> 64 -> 1 network with SiLU
// activations that learns the rest of the exact pair energy (the patch attraction).
// Other pair classes and bonded partners contribute 0 (their exact energy still enters
// the second stage).
//
// Features (12, invariant under rotations of the pair and under flipping either axis,
// which leaves PSC/CPSC energies unchanged), with r = c1 - c2 the FP32 minimum-image
// separation, a the axes, p the first patch directions, (s, t) the closest-point
// parameters and v = r + s a1 - t a2:
//   0 d                         6 p2 . unit(v - (v.a2) a2)
//   1 |r| / 4                   7 |s| / h1
//   2 |a1 . r^|                 8 |t| / h2
//   3 |a2 . r^|                 9 p1 . p2
//   4 (a1 . a2) sgn(a1.r) sgn(a2.r)   10 type code of particle 1
//   5 p1 . unit(-v + (v.a1) a1) 11 type code of particle 2
// input 12 is the constant 1 (the first layer's bias), inputs 13-15 are 0.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace scg {

constexpr int kFeat = 16;          // MLP input width (12 features, bias input, 3 zero pads)
constexpr int kHidden = 64;
// FP32 master parameters, flat
constexpr int kOffW1 = 0;                          // [16][64], row 12 = first-layer bias
constexpr int kOffW2 = kOffW1 + kFeat * kHidden;   // [64][64]
constexpr int kOffB2 = kOffW2 + kHidden * kHidden;
constexpr int kOffW3 = kOffB2 + kHidden;           // [64][64]
constexpr int kOffB3 = kOffW3 + kHidden * kHidden;
constexpr int kOffW4 = kOffB3 + kHidden;           // [64]
constexpr int kOffB4 = kOffW4 + kHidden;
constexpr int kParams = kOffB4 + 1;                // 9409
constexpr int kParamsPad = 9412;

// BF16 operand fragments of mma.sync.m16n8k16 (B operand, "col" layout), one 32-lane
// block of uint2 per (k-tile, n-tile): lane (g = lane/4, q = lane%4) holds
// {B[16kt+2q][8nt+g], B[16kt+2q+1][8nt+g]} and {B[16kt+2q+8][8nt+g], B[16kt+2q+9][8nt+g]}.
struct MlpPacked {
    uint2 f1[8][32];          // W1       (K 16, N 64)
    uint2 f2[4][8][32];       // W2       (K 64, N 64)
    uint2 f3[4][8][32];       // W3
    uint2 f4[4][32];          // W4       (K 64, N 8, column 0 = W4)
    uint2 t2[4][8][32];       // W2^T     (backward of layer 2)
    uint2 t3[4][8][32];       // W3^T
    float b2[kHidden], b3[kHidden], w4[kHidden], b4, rcutS;
    float pad_[2];
};

__device__ __forceinline__ uint32_t packBf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float bf16Round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// D = A * B + C, m16n8k16, BF16 operands, FP32 accumulation.
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint2 b, const float (&c)[4]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%10,%11,%12,%13};\n"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y), "f"(c[0]), "f"(c[1]), "f"(c[2]),
          "f"(c[3]));
}

// SiLU with the fast exponential and division intrinsics: the network is trained and
// evaluated with this same function, so its approximation is part of the model.
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float siluGrad(float z) {
    float sg = __fdividef(1.0f, 1.0f + __expf(-z));
    return sg * (1.0f + z * (1.0f - sg));
}

// FP32 closest approach of two segments (centres r = c1 - c2 apart, unit axes u, v, half
// lengths h1, h2): line solution clamped, then alternating clamped minimisation.
// Returns |w|^2, w = r + s u - t v the vector between the closest points.
__device__ __forceinline__ float segClosestF(float3 r, float3 u, float3 v, float h1, float h2, float& s, float& t,
                                             float3& w) {
    float b = u.x * v.x + u.y * v.y + u.z * v.z;
    float d = u.x * r.x + u.y * r.y + u.z * r.z;
    float e = v.x * r.x + v.y * r.y + v.z * r.z;
    float den = 1.0f - b * b;
    s = den > 1e-6f ? (b * e - d) / den : 0.0f;
    s = fminf(fmaxf(s, -h1), h1);
    t = fminf(fmaxf(b * s + e, -h2), h2);
    s = fminf(fmaxf(b * t - d, -h1), h1);
    t = fminf(fmaxf(b * s + e, -h2), h2);
    w = make_float3(r.x + s * u.x - t * v.x, r.y + s * u.y - t * v.y, r.z + s * u.z - t * v.z);
    return w.x * w.x + w.y * w.y + w.z * w.z;
}

// FP32 minimum image of two wrapped FP32 box fractions, scaled by the box: c1 - c2.
__device__ __forceinline__ float3 pairVecF(float3 c1, float4 c2, float bx, float by, float bz) {
    float dx = c1.x - c2.x, dy = c1.y - c2.y, dz = c1.z - c2.z;
    dx -= rintf(dx); dy -= rintf(dy); dz -= rintf(dz);
    return make_float3(dx * bx, dy * by, dz * bz);
}

__device__ __forceinline__ float dotf(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Wrapped FP32 box fraction of an (unwrapped) FP64 box fraction.
__device__ __forceinline__ float frac32(double x) {
    double f = x - floor(x);
    float v = (float)f;
    return v >= 1.0f ? 0.0f : v;
}

// Type input of the surrogate: the compact type index scaled to [0, 1].
__device__ __forceinline__ float typeCode(int t, int ntypes) { return ntypes > 1 ? (float)t / (float)(ntypes - 1) : 0.0f; }

// Truncated WCA of the segment distance in FP32 (the repulsive part of the surrogate),
// clamped so that sums of overlapping pairs stay finite.
__device__ __forceinline__ float wca32(float d2, float sigma, float epsilon, float rcutwcaSq) {
    if (!(d2 < rcutwcaSq)) return 0.0f;
    float x = sigma * sigma / fmaxf(d2, 1e-12f);
    float x3 = x * x * x;
    float e = 4.0f * epsilon * (x3 * x3 - x3) + epsilon;
    return fminf(e, 1e30f);
}

// The 16 MLP inputs of pair (1, 2).  Returns the FP32 segment distance^2.
__device__ __forceinline__ float pairFeatures(float3 r, float3 a1, float3 p1, float h1, float tc1, float3 a2, float3 p2,
                                              float h2, float tc2, float* f) {
    float s, t;
    float3 w;
    float d2 = segClosestF(r, a1, a2, h1, h2, s, t, w);
    float d = sqrtf(d2);
    float rr = sqrtf(dotf(r, r));
    float inv = rr > 1e-12f ? 1.0f / rr : 0.0f;
    float ar1 = dotf(a1, r) * inv, ar2 = dotf(a2, r) * inv;
    float sg = (ar1 < 0.0f ? -1.0f : 1.0f) * (ar2 < 0.0f ? -1.0f : 1.0f);
    // directions towards the other particle, perpendicular to the own axis
    float wa1 = dotf(w, a1), wa2 = dotf(w, a2);
    float3 n1 = make_float3(-w.x + wa1 * a1.x, -w.y + wa1 * a1.y, -w.z + wa1 * a1.z);
    float3 n2 = make_float3(w.x - wa2 * a2.x, w.y - wa2 * a2.y, w.z - wa2 * a2.z);
    float l1 = sqrtf(dotf(n1, n1)), l2 = sqrtf(dotf(n2, n2));
    f[0] = d;
    f[1] = rr * 0.25f;
    f[2] = fabsf(ar1);
    f[3] = fabsf(ar2);
    f[4] = dotf(a1, a2) * sg;
    f[5] = l1 > 1e-6f ? dotf(p1, n1) / l1 : 0.0f;
    f[6] = l2 > 1e-6f ? dotf(p2, n2) / l2 : 0.0f;
    f[7] = h1 > 0.0f ? fabsf(s) / h1 : 0.0f;
    f[8] = h2 > 0.0f ? fabsf(t) / h2 : 0.0f;
    f[9] = dotf(p1, p2);
    f[10] = tc1;
    f[11] = tc2;
    f[12] = 1.0f;
    f[13] = 0.0f;
    f[14] = 0.0f;
    f[15] = 0.0f;
    return d2;
}

// A fragment (16 x 16, row major) of rows X[0..15][0..15] held in shared memory.
__device__ __forceinline__ void loadA16(const float (*X)[kFeat], uint32_t (&a)[4], int lane) {
    const int g = lane >> 2, q = lane & 3;
    a[0] = packBf16(X[g][2 * q], X[g][2 * q + 1]);
    a[1] = packBf16(X[g + 8][2 * q], X[g + 8][2 * q + 1]);
    a[2] = packBf16(X[g][2 * q + 8], X[g][2 * q + 9]);
    a[3] = packBf16(X[g + 8][2 * q + 8], X[g + 8][2 * q + 9]);
}

// The C fragments of n-tiles 2kt and 2kt+1 are the A fragment of k-tile kt of the next
// layer (same lane owns the same rows and columns).
__device__ __forceinline__ void cToA(const float (&c0)[4], const float (&c1)[4], uint32_t (&a)[4]) {
    a[0] = packBf16(c0[0], c0[1]);
    a[1] = packBf16(c0[2], c0[3]);
    a[2] = packBf16(c1[0], c1[1]);
    a[3] = packBf16(c1[2], c1[3]);
}

// One hidden layer 64 -> 64: z = h W + b (C layout, 8 n-tiles), h given as 4 A fragments.
__device__ __forceinline__ void hiddenLayer(const uint2 (*F)[8][32], const float* bias, const uint32_t (&h)[4][4],
                                            float (&z)[8][4], int lane) {
    const int q = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float b0 = bias[nt * 8 + 2 * q], b1 = bias[nt * 8 + 2 * q + 1];
        float c[4] = {b0, b1, b0, b1};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) mma16816(c, h[kt], F[kt][nt][lane], c);
#pragma unroll
        for (int e = 0; e < 4; ++e) z[nt][e] = c[e];
    }
}

// Forward pass of one warp over 16 rows X (shared memory).  On return lanes with
// lane % 4 == 0 hold the outputs of rows lane/4 (y0) and lane/4 + 8 (y1).
__device__ __forceinline__ void mlpForward16(const MlpPacked* __restrict__ P, const float (*X)[kFeat], float& y0,
                                             float& y1) {
    const int lane = threadIdx.x & 31;
    uint32_t a0[4];
    loadA16(X, a0, lane);
    float z[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        mma16816(c, a0, P->f1[nt][lane], c);
#pragma unroll
        for (int e = 0; e < 4; ++e) z[nt][e] = silu(c[e]);
    }
    uint32_t h[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) cToA(z[2 * kt], z[2 * kt + 1], h[kt]);
    hiddenLayer(P->f2, P->b2, h, z, lane);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) z[nt][e] = silu(z[nt][e]);
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) cToA(z[2 * kt], z[2 * kt + 1], h[kt]);
    hiddenLayer(P->f3, P->b3, h, z, lane);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) z[nt][e] = silu(z[nt][e]);
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) cToA(z[2 * kt], z[2 * kt + 1], h[kt]);
    const float b4 = P->b4;
    float c[4] = {b4, 0.0f, b4, 0.0f};
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) mma16816(c, h[kt], P->f4[kt][lane], c);
    y0 = c[0];
    y1 = c[2];
}

}  // namespace scg
