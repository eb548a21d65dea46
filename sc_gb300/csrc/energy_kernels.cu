// energy_kernels.cu -- pair, one-particle and total energies (the TotalE interface of
// scOOP/mc/totalenergycalculator.h:136-297) over all particles, FP64.
//
// These are the exact, order-independent reference calls: every pair is tested
// with the PairE prefilter, so they serve arbitrary configurations (any box,
// any N) and anchor the parity tests.  The sweep kernels use cell lists instead.

#include "kernels.h"
#include "pair_energy.cuh"

namespace scg {

namespace {

__device__ __forceinline__ PView viewOf(const DevState& s, int j, const TrialSlot* trial, int trialIndex) {
    PView v;
    if (trial && j == trialIndex) {
        v.pos = mk(trial->pos.x, trial->pos.y, trial->pos.z);
        v.dir = mk(trial->dir.x, trial->dir.y, trial->dir.z);
        v.patch = &trial->patch;
        v.type = (int)trial->pos.w;
    } else {
        double4_32a p = s.pos[j];
        double4_32a d = s.dir[j];
        v.pos = mk(p.x, p.y, p.z);
        v.dir = mk(d.x, d.y, d.z);
        v.patch = &s.patch[j];
        v.type = (int)p.w;
    }
    v.index = j;
    v.molType = s.mol[j].x;
    return v;
}

__device__ __forceinline__ DevCtx ctxOf(const DevState& s, const DevTables& t) {
    DevCtx c;
    c.params = t.params;
    c.mols = t.mols;
    c.ntypes = t.ntypes;
    c.n = s.n;
    c.sqmaxcut = t.sqmaxcut;
    return c;
}

// Deterministic block sum (fixed shuffle tree, then fixed order over warps).
template <int BLOCK>
__device__ __forceinline__ double blockSum(double v) {
    __shared__ double warpSums[BLOCK / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warpSums[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < BLOCK / 32; ++k) r += warpSums[k];
    __syncthreads();
    return r;
}

__global__ void kPairBatch(DevState s, DevTables t, int npairs, const int* __restrict__ I, const int* __restrict__ J,
                           double* E, unsigned* bits, double* dsq) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npairs) return;
    int i = I[k], j = J[k];
    if (i < 0 || j < 0 || i >= s.n || j >= s.n) {   // checked on the host too
        E[k] = 0.0; bits[k] = 0xffffffffu; dsq[k] = -1.0;
        return;
    }
    DevCtx c = ctxOf(s, t);
    double3 box = mk(s.box[0], s.box[1], s.box[2]);
    PView a = viewOf(s, i, nullptr, -1), b = viewOf(s, j, nullptr, -1);
    Con con = makeCon(c, i, s.mol[i]);
    unsigned bb;
    double d;
    E[k] = pairEnergy(c, a, b, con, box, &bb, &d);
    bits[k] = bb;
    dsq[k] = d;
}

constexpr int kOneBlock = 256;

__global__ void __launch_bounds__(kOneBlock) kOneToAll(DevState s, DevTables t, const int* __restrict__ targets,
                                                      const TrialSlot* trial, double* out) {
    int target = targets[blockIdx.x];
    DevCtx c = ctxOf(s, t);
    double3 box = mk(s.box[0], s.box[1], s.box[2]);
    int trialIdx = (trial && blockIdx.x == 0) ? target : -1;
    PView a = viewOf(s, target, trialIdx >= 0 ? trial : nullptr, trialIdx);
    Con con = makeCon(c, target, s.mol[target]);
    double sum = 0.0;
    for (int j = threadIdx.x; j < s.n; j += kOneBlock) {
        if (j == target) continue;
        PView b = viewOf(s, j, nullptr, -1);
        unsigned bb;
        double d;
        sum += pairEnergy(c, a, b, con, box, &bb, &d);
    }
    double r = blockSum<kOneBlock>(sum);
    if (threadIdx.x == 0) out[blockIdx.x] = r;
}

constexpr int kAllBlock = 128;

// Thread i sums PairE(i, j, conlist(i)) over j < i (allToAll's part1 = i > j).
__global__ void __launch_bounds__(kAllBlock) kAllToAll(DevState s, DevTables t, const double* boxOverride, double* partial) {
    DevCtx c = ctxOf(s, t);
    const double* bx = boxOverride ? boxOverride : s.box;
    double3 box = mk(bx[0], bx[1], bx[2]);
    double sum = 0.0;
    // interleave rows so that blocks get balanced work: rows i and n-1-i
    int half = (s.n + 1) / 2;
    int r = blockIdx.x * kAllBlock + threadIdx.x;
    if (r < half) {
        int rows[2] = {r, s.n - 1 - r};
        for (int q = 0; q < 2; ++q) {
            int i = rows[q];
            if (q == 1 && i == rows[0]) break;
            PView a = viewOf(s, i, nullptr, -1);
            Con con = makeCon(c, i, s.mol[i]);
            for (int j = 0; j < i; ++j) {
                PView b = viewOf(s, j, nullptr, -1);
                unsigned bb;
                double d;
                sum += pairEnergy(c, a, b, con, box, &bb, &d);
            }
        }
    }
    double v = blockSum<kAllBlock>(sum);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

// Updater::alignmentOrder (scOOP/mc/updater.cpp:466-481): sum of dir_i . dir_j over pairs
// closer than 1.5 (minimum image, centres); thread per row pair (i, n-1-i), j > i.
__global__ void __launch_bounds__(kAllBlock) kAlignment(DevState s, double* partial) {
    double3 box = mk(s.box[0], s.box[1], s.box[2]);
    double sum = 0.0;
    int half = (s.n + 1) / 2;
    int r = blockIdx.x * kAllBlock + threadIdx.x;
    if (r < half) {
        int rows[2] = {r, s.n - 1 - r};
        for (int q = 0; q < 2; ++q) {
            int i = rows[q];
            if (q == 1 && i == rows[0]) break;
            double4_32a pi = s.pos[i], di = s.dir[i];
            for (int j = i + 1; j < s.n; ++j) {
                double4_32a pj = s.pos[j];
                double3 rc = imageVec(mk(pi.x, pi.y, pi.z), mk(pj.x, pj.y, pj.z), box);
                if (dot3(rc, rc) < 1.5 * 1.5) {
                    double4_32a dj = s.dir[j];
                    sum += di.x * dj.x + di.y * dj.y + di.z * dj.z;
                }
            }
        }
    }
    double v = blockSum<kAllBlock>(sum);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

__global__ void kFinalSum(const double* partial, int n, double* out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double r = 0.0;
        for (int k = 0; k < n; ++k) r += partial[k];
        *out = r;
    }
}

__global__ void __launch_bounds__(kOneBlock) kMolToOthers(DevState s, DevTables t, int first, int size, double* out) {
    DevCtx c = ctxOf(s, t);
    double3 box = mk(s.box[0], s.box[1], s.box[2]);
    Con con = emptyCon(c);
    double sum = 0.0;
    int others = s.n - size;
    for (int q = 0; q < size; ++q) {
        PView a = viewOf(s, first + q, nullptr, -1);
        for (int k = threadIdx.x; k < others; k += kOneBlock) {
            int j = k < first ? k : k + size;
            PView b = viewOf(s, j, nullptr, -1);
            unsigned bb;
            double d;
            sum += pairEnergy(c, a, b, con, box, &bb, &d);
        }
    }
    double r = blockSum<kOneBlock>(sum);
    if (threadIdx.x == 0) *out = r;
}

}  // namespace

cudaError_t launchPairBatch(const DevState& s, const DevTables& t, int npairs, const int* I, const int* J, double* E,
                            unsigned* bits, double* dsq, cudaStream_t st) {
    if (npairs <= 0) return cudaSuccess;
    kPairBatch<<<(npairs + 127) / 128, 128, 0, st>>>(s, t, npairs, I, J, E, bits, dsq);
    return cudaGetLastError();
}

cudaError_t launchOneToAll(const DevState& s, const DevTables& t, int ntargets, const int* targets,
                           const TrialSlot* trial, double* out, cudaStream_t st) {
    if (ntargets <= 0) return cudaSuccess;
    kOneToAll<<<ntargets, kOneBlock, 0, st>>>(s, t, targets, trial, out);
    return cudaGetLastError();
}

int allToAllBlocks(int n) { return ((n + 1) / 2 + kAllBlock - 1) / kAllBlock; }

// Second-moment sums of the axes of the spherocylinders (geotype < SP): out[0] their count,
// out[1..6] the sums of xx, yy, zz, xy, xz, yz.  One CTA; every thread sums a fixed strided
// subset, then a fixed tree: the result does not depend on scheduling.
__global__ void __launch_bounds__(256) kAxisMoments(DevState s, DevTables t, double* out) {
    __shared__ double red[7][256];
    double m[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < s.n; i += 256) {
        const int ty = (int)s.pos[i].w;
        if (t.params[ty * t.ntypes + ty].geotype[0] >= SP) continue;
        const double4_32a d = s.dir[i];
        m[0] += 1.0;
        m[1] += d.x * d.x; m[2] += d.y * d.y; m[3] += d.z * d.z;
        m[4] += d.x * d.y; m[5] += d.x * d.z; m[6] += d.y * d.z;
    }
    for (int k = 0; k < 7; ++k) red[k][threadIdx.x] = m[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < 7; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 7) out[threadIdx.x] = red[threadIdx.x][0];
}

cudaError_t launchAxisMoments(const DevState& s, const DevTables& t, double* out, cudaStream_t st) {
    kAxisMoments<<<1, 256, 0, st>>>(s, t, out);
    return cudaGetLastError();
}

cudaError_t launchAlignment(const DevState& s, double* partial, int npartial, double* out, cudaStream_t st) {
    int nb = allToAllBlocks(s.n);
    if (nb > npartial) return cudaErrorInvalidValue;
    if (nb > 0) kAlignment<<<nb, kAllBlock, 0, st>>>(s, partial);
    kFinalSum<<<1, 32, 0, st>>>(partial, nb, out);
    return cudaGetLastError();
}

cudaError_t launchAllToAll(const DevState& s, const DevTables& t, const double* boxOverride, double* partial,
                           int npartial, double* out, cudaStream_t st) {
    int nb = allToAllBlocks(s.n);
    if (nb > npartial) return cudaErrorInvalidValue;
    if (nb > 0) kAllToAll<<<nb, kAllBlock, 0, st>>>(s, t, boxOverride, partial);
    kFinalSum<<<1, 32, 0, st>>>(partial, nb, out);
    return cudaGetLastError();
}

cudaError_t launchMolToOthers(const DevState& s, const DevTables& t, int first, int size, double* out, cudaStream_t st) {
    kMolToOthers<<<1, kOneBlock, 0, st>>>(s, t, first, size, out);
    return cudaGetLastError();
}

}  // namespace scg
