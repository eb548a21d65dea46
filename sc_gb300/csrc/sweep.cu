// sweep.cu -- the on-device Metropolis move loop (Updater::simulate, scOOP/mc/updater.cpp:45-389).
//
// One sweep = N attempted single-particle moves, run as a checkerboard over a cell
// list so that moves in different cells proceed concurrently without changing the
// stationary distribution:
//   * cells are at least maxcut (= sqrt(sqmaxcut), the PairE prefilter range) wide,
//     so every particle that can interact with a particle of a cell lies in that cell
//     or one of its 26 neighbours;
//   * each sweep shifts the cell grid by a random offset, rebuilds the cell list
//     (counting sort), and visits the 2x2x2 colour classes in random order; cells of
//     one colour are never neighbours, so their moves are independent;
//   * a cell performs as many moves as it holds particles, each on a randomly chosen
//     particle of the cell; a displacement that would leave the cell is rejected
//     (this keeps the cells independent and the move set symmetric);
//   * proposals are those of MoveCreator::partDisplace / partRotate
//     (scOOP/mc/movecreator.cpp:947-1028): a displacement of fixed length transmx in
//     a uniformly random direction, or Particle::pscRotate by angle rot_angle*u about
//     a random axis; spheres only move.  Acceptance is MoveCreator::moveTry
//     (movecreator.h:175-187).
//   * the isotropic volume move of ptype 1 (movecreator.cpp:390-421) runs after a sweep
//     on the device: total energy of the rescaled box over the cell list, then the
//     reference's acceptance rule.
// All random numbers are Philox draws keyed by (seed, sweep, cell, move), so a run is
// reproducible and independent of scheduling.
//
// One CTA owns one active cell.  For every move its threads scan the candidate list
// (the cell and its neighbours, staged in shared memory), apply the cutoff prefilter in
// FP64, compact the surviving (particle, old/new) pairs into a shared queue with a
// deterministic block scan, evaluate the queue one pair per thread and reduce the old
// and new energies in a fixed order.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "pair_energy.cuh"
#include "philox.cuh"
#include "sc_context.h"

namespace scg {

namespace {

constexpr int kMoveThreads = 128;
constexpr int kCellCap = 256;        // particles per cell
constexpr int kCandCap = 1536;       // candidates staged in shared memory
constexpr int kQueueCap = 1024;      // pair queue entries
constexpr int kTotThreads = 128;

enum Ctr { C_ACC_T, C_REJ_T, C_ACC_R, C_REJ_R, C_ACC_V, C_REJ_V, C_VOL_CONSTR, C_TESTED, C_EVAL, C_CELL_REJ, C_MOVES,
           C_COUNT };
enum ErrBit { E_CELL_OVERFLOW = 1, E_PARTNER_FAR = 2, E_GRID = 4 };

struct Grid {
    int nc[3];
    int p[3];         // colours per dimension (1 or 2)
    int ncells;
    int nactive;      // cells per colour
    int ncolours;
    double maxcut;
};

// Per-sweep control block, device resident (so that a sweep can be replayed as a graph).
struct Control {
    unsigned long long sweep;
    double shift[3];      // grid offset, box fractions
    int perm[8];          // colour order
    double psch;          // volume move: edge change
    int volValid;         // trial box keeps cells >= maxcut
    int pad_;
    double trialBox[3];
    double energy;        // running total energy
    double energyCheck;   // last exact total energy
    double maxDrift;
};

struct SweepArgs {
    DevState s;
    DevTables t;
    Grid g;
    Control* ctl;
    int* cellStart;
    int* cellCount;
    int* cellCursor;
    int* cellIdx;
    int* cellOf;
    double* cellDE;
    double* partial;      // total-energy block sums
    unsigned long long* counters;
    int* err;
    uint64_t seed;
    double temper, press;
    double rotAngle;
    double edgeMx;
    double trans[MAX_DEV_TYPES];
    int geo[MAX_DEV_TYPES];
};

__device__ __forceinline__ int wrapCell(double x, double shift, int nc) {
    double f = x - floor(x);
    f += shift;
    if (f >= 1.0) f -= 1.0;
    int c = (int)(f * nc);
    return c >= nc ? nc - 1 : (c < 0 ? 0 : c);
}

// Offsets of the neighbour cells along one dimension: each distinct cell once.
__device__ __forceinline__ int neighbourOffsets(int nc, int* off) {
    if (nc == 1) { off[0] = 0; return 1; }
    if (nc == 2) { off[0] = 0; off[1] = 1; return 2; }
    off[0] = -1; off[1] = 0; off[2] = 1;
    return 3;
}

__global__ void kBeginSweep(SweepArgs a, int volumeDue) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Control& c = *a.ctl;
    Stream r(a.seed, 0xFFFFFFF0u, (uint32_t)c.sweep, (uint32_t)(c.sweep >> 32));
    for (int d = 0; d < 3; ++d) c.shift[d] = r.next() / a.g.nc[d];
    int n = a.g.ncolours;
    for (int k = 0; k < n; ++k) c.perm[k] = k;
    for (int k = n - 1; k > 0; --k) {      // Fisher-Yates
        int j = (int)(r.next() * (k + 1));
        if (j > k) j = k;
        int tmp = c.perm[k]; c.perm[k] = c.perm[j]; c.perm[j] = tmp;
    }
    c.volValid = 0;
    if (volumeDue) {
        c.psch = a.edgeMx * (r.next() - 0.5);
        bool ok = true;
        for (int d = 0; d < 3; ++d) {
            c.trialBox[d] = a.s.box[d] + c.psch;
            if (!(c.trialBox[d] > 0.0) || c.trialBox[d] / a.g.nc[d] < a.g.maxcut) ok = false;
        }
        c.volValid = ok ? 1 : 0;
    }
}

__global__ void kAssign(SweepArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.s.n) return;
    const Control& c = *a.ctl;
    double4_32a p = a.s.pos[i];
    int cx = wrapCell(p.x, c.shift[0], a.g.nc[0]);
    int cy = wrapCell(p.y, c.shift[1], a.g.nc[1]);
    int cz = wrapCell(p.z, c.shift[2], a.g.nc[2]);
    int cell = (cz * a.g.nc[1] + cy) * a.g.nc[0] + cx;
    a.cellOf[i] = cell;
    atomicAdd(&a.cellCount[cell], 1);
}

__global__ void kScan(SweepArgs a) {
    // single block: exclusive scan of the cell counts
    __shared__ int warpTot[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = 0; base < a.g.ncells; base += blockDim.x) {
        int k = base + threadIdx.x;
        int v = k < a.g.ncells ? a.cellCount[k] : 0;
        if (v > kCellCap) atomicOr(a.err, E_CELL_OVERFLOW);
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warpTot[w] = incl;
        __syncthreads();
        int woff = 0, tot = 0;
        for (int q = 0; q < nw; ++q) { if (q < w) woff += warpTot[q]; tot += warpTot[q]; }
        if (k < a.g.ncells) {
            a.cellStart[k] = carry + woff + incl - v;
            a.cellCursor[k] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void kScatter(SweepArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.s.n) return;
    int cell = a.cellOf[i];
    int slot = a.cellStart[cell] + atomicAdd(&a.cellCursor[cell], 1);
    a.cellIdx[slot] = i;
}

// Orders each cell's particles by index (deterministic lists whatever the atomics did).
__global__ void kSortCells(SweepArgs a) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.g.ncells) return;
    int s = a.cellStart[c], n = a.cellCount[c];
    int* v = a.cellIdx + s;
    for (int i = 1; i < n; ++i) {
        int x = v[i], j = i - 1;
        while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; --j; }
        v[j + 1] = x;
    }
}

struct BlockScan {
    int warpTot[kMoveThreads / 32];
};

// Exclusive scan of v over the block; returns the offset, writes the total.
__device__ __forceinline__ int blockExclusiveScan(int v, int& total, BlockScan& sh) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) sh.warpTot[w] = incl;
    __syncthreads();
    int woff = 0;
    total = 0;
#pragma unroll
    for (int q = 0; q < kMoveThreads / 32; ++q) {
        int t = sh.warpTot[q];
        if (q < w) woff += t;
        total += t;
    }
    __syncthreads();
    return woff + incl - v;
}

// Fixed-order block sum of two doubles; result valid in thread 0.
__device__ __forceinline__ void blockSum2(double& x, double& y, double (*sh)[2]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, o);
        y += __shfl_down_sync(0xffffffffu, y, o);
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sh[w][0] = x; sh[w][1] = y; }
    __syncthreads();
    if (threadIdx.x == 0) {
        x = 0.0; y = 0.0;
        for (int q = 0; q < kMoveThreads / 32; ++q) { x += sh[q][0]; y += sh[q][1]; }
    }
    __syncthreads();
}

struct MoveShared {
    int list[kCellCap];
    int cand[kCandCap];
    int queue[kQueueCap];
    int nbCell[27];
    int nNb;
    int nCand;
    // current proposal
    int target, displace, skip, partners[4], nPartners;
    double umet;
    double npos[3], ndir[3];
    PatchSet npatch;
    BlockScan scan;
    double red[kMoveThreads / 32][2];
};

__device__ __forceinline__ void randomUnitSphere(Stream& r, double& x, double& y, double& z) {
    // Vector::randomUnitSphere (scOOP/structures/Vector.h:190-205)
    double a, xi1, xi2;
    do {
        xi1 = 1.0 - 2.0 * r.next();
        xi2 = 1.0 - 2.0 * r.next();
        a = xi1 * xi1 + xi2 * xi2;
    } while (a > 1.0);
    double b = 2.0 * sqrt(1.0 - a);
    x = xi1 * b; y = xi2 * b; z = 1.0 - 2.0 * a;
}

// Particle::pscRotate (scOOP/structures/particle.h:182-272) followed by the
// re-orthogonalisation of patchdir[0] in partRotate (movecreator.cpp:1007).
__device__ void pscRotate(double* dir, PatchSet& ps, int g, double angle, double ax, double ay, double az, bool positive) {
    double vc = cos(angle);
    double vs = positive ? sqrt(1.0 - vc * vc) : -sqrt(1.0 - vc * vc);
    double qw = vc, qx = ax * vs, qy = ay * vs, qz = az * vs;
    double t2 = qw * qx, t3 = qw * qy, t4 = qw * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
           t9 = qy * qz, t10 = -qz * qz;
    double d1 = t8 + t10, d2 = t6 - t4, d3 = t3 + t7, d4 = t4 + t6, d5 = t5 + t10, d6 = t9 - t2, d7 = t7 - t3,
           d8 = t2 + t9, d9 = t5 + t8;
    auto rot = [&](double* v) {
        double nx = 2.0 * (d1 * v[0] + d2 * v[1] + d3 * v[2]) + v[0];
        double ny = 2.0 * (d4 * v[0] + d5 * v[1] + d6 * v[2]) + v[1];
        double nz = 2.0 * (d7 * v[0] + d8 * v[1] + d9 * v[2]) + v[2];
        v[0] = nx; v[1] = ny; v[2] = nz;
    };
    rot(dir);
    if (g != SCN && g != SCA) {
        int m = isTwoPatch(g) ? 2 : 1;
        for (int k = 0; k < m; ++k) { rot(ps.pd[k]); rot(ps.ps[2 * k]); rot(ps.ps[2 * k + 1]); }
    }
    if (isChiral(g)) {
        int m = (g == TCHPSC || g == TCHCPSC) ? 2 : 1;
        for (int k = 0; k < m; ++k) rot(ps.ch[k]);
    }
    double dp = ps.pd[0][0] * dir[0] + ps.pd[0][1] * dir[1] + ps.pd[0][2] * dir[2];
    ps.pd[0][0] -= dp * dir[0]; ps.pd[0][1] -= dp * dir[1]; ps.pd[0][2] -= dp * dir[2];
}

__device__ __forceinline__ PView viewAt(const DevState& s, int j) {
    PView v;
    double4_32a p = s.pos[j];
    double4_32a d = s.dir[j];
    v.pos = mk(p.x, p.y, p.z);
    v.dir = mk(d.x, d.y, d.z);
    v.patch = &s.patch[j];
    v.type = (int)p.w;
    v.index = j;
    v.molType = 0;
    return v;
}

__global__ void __launch_bounds__(kMoveThreads) kColour(SweepArgs a, int phase) {
    __shared__ MoveShared sh;
    const Control& ctl = *a.ctl;
    const Grid& g = a.g;
    int colour = ctl.perm[phase];
    int ox = colour % g.p[0], oy = (colour / g.p[0]) % g.p[1], oz = colour / (g.p[0] * g.p[1]);
    int ax = g.nc[0] / g.p[0], ay = g.nc[1] / g.p[1];
    int bx = blockIdx.x % ax, by = (blockIdx.x / ax) % ay, bz = blockIdx.x / (ax * ay);
    int cx = ox + g.p[0] * bx, cy = oy + g.p[1] * by, cz = oz + g.p[2] * bz;
    int cell = (cz * g.nc[1] + cy) * g.nc[0] + cx;
    int cnt = a.cellCount[cell];
    if (cnt == 0 || cnt > kCellCap) return;
    const int tid = threadIdx.x;
    const int* idx = a.cellIdx;
    for (int k = tid; k < cnt; k += kMoveThreads) sh.list[k] = idx[a.cellStart[cell] + k];
    if (tid == 0) {
        int offx[3], offy[3], offz[3];
        int nx = neighbourOffsets(g.nc[0], offx), ny = neighbourOffsets(g.nc[1], offy), nz = neighbourOffsets(g.nc[2], offz);
        int nn = 0;
        for (int qz = 0; qz < nz; ++qz)
            for (int qy = 0; qy < ny; ++qy)
                for (int qx = 0; qx < nx; ++qx) {
                    int x = (cx + offx[qx] + g.nc[0]) % g.nc[0];
                    int y = (cy + offy[qy] + g.nc[1]) % g.nc[1];
                    int z = (cz + offz[qz] + g.nc[2]) % g.nc[2];
                    sh.nbCell[nn++] = (z * g.nc[1] + y) * g.nc[0] + x;
                }
        sh.nNb = nn;
        int m = 0;
        for (int q = 0; q < nn; ++q) m += a.cellCount[sh.nbCell[q]];
        sh.nCand = m;
    }
    __syncthreads();
    const int nCand = sh.nCand;
    const bool staged = nCand <= kCandCap;
    if (staged) {
        // flatten the candidate list (cells in order, particles by index)
        int base = 0;
        for (int q = 0; q < sh.nNb; ++q) {
            int c2 = sh.nbCell[q], n2 = a.cellCount[c2], s2 = a.cellStart[c2];
            for (int k = tid; k < n2; k += kMoveThreads) sh.cand[base + k] = idx[s2 + k];
            base += n2;
        }
    }
    __syncthreads();

    DevCtx c;
    c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = a.s.n; c.sqmaxcut = a.t.sqmaxcut;
    const double3 box = mk(a.s.box[0], a.s.box[1], a.s.box[2]);
    double dECell = 0.0;
    unsigned long long nAccT = 0, nRejT = 0, nAccR = 0, nRejR = 0, nTested = 0, nEval = 0, nCellRej = 0;

    for (int m = 0; m < cnt; ++m) {
        if (tid == 0) {
            Stream r(a.seed, (uint32_t)cell, (uint32_t)m, (uint32_t)ctl.sweep ^ ((uint32_t)(ctl.sweep >> 32) << 20));
            int t = sh.list[min((int)(r.next() * cnt), cnt - 1)];
            double4_32a p = a.s.pos[t];
            double4_32a d = a.s.dir[t];
            int type = (int)p.w;
            int geo = a.geo[type];
            bool displace = (r.next() < 0.5) || geo >= SP;
            sh.target = t;
            sh.displace = displace;
            sh.skip = 0;
            if (displace) {
                double x, y, z;
                randomUnitSphere(r, x, y, z);
                double mx = a.trans[type];
                x *= mx / box.x; y *= mx / box.y; z *= mx / box.z;
                sh.npos[0] = p.x + x; sh.npos[1] = p.y + y; sh.npos[2] = p.z + z;
                sh.ndir[0] = d.x; sh.ndir[1] = d.y; sh.ndir[2] = d.z;
                int nx = wrapCell(sh.npos[0], ctl.shift[0], g.nc[0]);
                int ny = wrapCell(sh.npos[1], ctl.shift[1], g.nc[1]);
                int nz = wrapCell(sh.npos[2], ctl.shift[2], g.nc[2]);
                if (nx != cx || ny != cy || nz != cz) sh.skip = 1;     // would leave the cell
            } else {
                double angle = a.rotAngle * r.next();
                double x, y, z;
                randomUnitSphere(r, x, y, z);
                bool positive = r.next() < 0.5;
                sh.npos[0] = p.x; sh.npos[1] = p.y; sh.npos[2] = p.z;
                sh.ndir[0] = d.x; sh.ndir[1] = d.y; sh.ndir[2] = d.z;
                sh.npatch = a.s.patch[t];
                pscRotate(sh.ndir, sh.npatch, geo, angle, x, y, z, positive);
            }
            sh.umet = r.next();
            // bonded partners are evaluated explicitly; they must sit in this or a neighbour cell
            int4 mi = a.s.mol[t];
            Con con = makeCon(c, t, mi);
            int np = 0;
            for (int q = 0; q < 4; ++q) {
                int j = con.idx[q];
                if (j < 0) continue;
                bool near = false;
                int cj = a.cellOf[j];
                for (int w = 0; w < sh.nNb; ++w) near |= (sh.nbCell[w] == cj);
                if (!near) { atomicOr(a.err, E_PARTNER_FAR); sh.skip = 1; }
                sh.partners[np++] = j;
            }
            sh.nPartners = np;
        }
        __syncthreads();
        const int t = sh.target;
        if (sh.skip) {
            if (tid == 0) { if (sh.displace) { ++nRejT; ++nCellRej; } else ++nRejR; }
            __syncthreads();
            continue;
        }
        const bool displace = sh.displace;
        const int np = sh.nPartners;
        int partners[4] = {-1, -1, -1, -1};
        for (int q = 0; q < np; ++q) partners[q] = sh.partners[q];
        double4_32a op4 = a.s.pos[t];
        double4_32a od4 = a.s.dir[t];
        PView oldV;
        oldV.pos = mk(op4.x, op4.y, op4.z);
        oldV.dir = mk(od4.x, od4.y, od4.z);
        oldV.patch = &a.s.patch[t];
        oldV.type = (int)op4.w;
        oldV.index = t;
        oldV.molType = 0;
        PView newV = oldV;
        newV.pos = mk(sh.npos[0], sh.npos[1], sh.npos[2]);
        newV.dir = mk(sh.ndir[0], sh.ndir[1], sh.ndir[2]);
        if (!displace) newV.patch = &sh.npatch;
        Con con = makeCon(c, t, a.s.mol[t]);

        double eOld = 0.0, eNew = 0.0;
        int qn = 0;
        // bonded partners: both configurations, whatever the distance
        if (tid < np) {
            PView b = viewAt(a.s, partners[tid]);
            unsigned bb; double dd;
            eOld += pairEnergy(c, oldV, b, con, box, &bb, &dd);
            eNew += pairEnergy(c, newV, b, con, box, &bb, &dd);
        }
        auto flush = [&](int count) {
            for (int e = tid; e < count; e += kMoveThreads) {
                int q = sh.queue[e];
                int j = q >> 1;
                PView b = viewAt(a.s, j);
                unsigned bb; double dd;
                if (q & 1) eNew += pairEnergy(c, newV, b, con, box, &bb, &dd);
                else eOld += pairEnergy(c, oldV, b, con, box, &bb, &dd);
            }
            __syncthreads();
        };
        for (int base = 0; base < nCand; base += kMoveThreads) {
            int k = base + tid;
            int flags = 0, j = -1;
            if (k < nCand) {
                if (staged) j = sh.cand[k];
                else {
                    int rem = k;
                    for (int q = 0; q < sh.nNb; ++q) {
                        int n2 = a.cellCount[sh.nbCell[q]];
                        if (rem < n2) { j = idx[a.cellStart[sh.nbCell[q]] + rem]; break; }
                        rem -= n2;
                    }
                }
                bool partner = (j == partners[0] || j == partners[1] || j == partners[2] || j == partners[3]);
                if (j != t && !partner) {
                    double4_32a pj = a.s.pos[j];
                    double3 pp = mk(pj.x, pj.y, pj.z);
                    double3 r0 = imageVec(oldV.pos, pp, box);
                    bool pass0 = !(dot3(r0, r0) > c.sqmaxcut);
                    bool pass1 = pass0;
                    if (displace) {
                        double3 r1 = imageVec(newV.pos, pp, box);
                        pass1 = !(dot3(r1, r1) > c.sqmaxcut);
                    }
                    flags = (pass0 ? 1 : 0) | (pass1 ? 2 : 0);
                }
            }
            int total;
            int off = blockExclusiveScan(__popc(flags), total, sh.scan);
            if (flags & 1) sh.queue[qn + off++] = j << 1;
            if (flags & 2) sh.queue[qn + off] = (j << 1) | 1;
            qn += total;
            __syncthreads();
            if (qn > kQueueCap - 2 * kMoveThreads) {
                flush(qn);
                nEval += qn;
                qn = 0;
            }
        }
        flush(qn);
        nEval += qn + 2 * np;
        nTested += (unsigned long long)nCand * (displace ? 2 : 1);
        blockSum2(eOld, eNew, sh.red);
        if (tid == 0) {
            // MoveCreator::moveTry (movecreator.h:175-187)
            bool accept = (eNew <= eOld) || (exp(-1.0 * (eNew - eOld) / a.temper) > sh.umet);
            if (accept) {
                a.s.pos[t] = make_double4_32a(sh.npos[0], sh.npos[1], sh.npos[2], op4.w);
                if (!displace) {
                    a.s.dir[t] = make_double4_32a(sh.ndir[0], sh.ndir[1], sh.ndir[2], od4.w);
                    a.s.patch[t] = sh.npatch;
                }
                dECell += eNew - eOld;
                if (displace) ++nAccT; else ++nAccR;
            } else {
                if (displace) ++nRejT; else ++nRejR;
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        a.cellDE[cell] = dECell;
        atomicAdd(&a.counters[C_ACC_T], nAccT);
        atomicAdd(&a.counters[C_REJ_T], nRejT);
        atomicAdd(&a.counters[C_ACC_R], nAccR);
        atomicAdd(&a.counters[C_REJ_R], nRejR);
        atomicAdd(&a.counters[C_CELL_REJ], nCellRej);
        atomicAdd(&a.counters[C_MOVES], (unsigned long long)cnt);
    }
    // per-thread pair counters
    unsigned long long tested = tid == 0 ? nTested : 0ull, ev = tid == 0 ? nEval : 0ull;
    if (tid == 0) {
        atomicAdd(&a.counters[C_TESTED], tested);
        atomicAdd(&a.counters[C_EVAL], ev);
    }
}

// Adds the cells' energy changes of this sweep, in a fixed order.
__global__ void kEndSweep(SweepArgs a) {
    __shared__ double ws[32];
    double v = 0.0;
    for (int k = threadIdx.x; k < a.g.ncells; k += blockDim.x) v += a.cellDE[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += ws[q];
        a.ctl->energy += s;
        a.ctl->sweep += 1;
    }
}

// Total energy over the cell list: thread i adds PairE(i, j, conlist(i)) for j < i
// (allToAll's pair orientation, totalenergycalculator.h:502-521).
__global__ void __launch_bounds__(kTotThreads) kTotalEnergy(SweepArgs a, int useTrialBox) {
    __shared__ double ws[kTotThreads / 32];
    const Control& ctl = *a.ctl;
    int i = blockIdx.x * kTotThreads + threadIdx.x;
    double sum = 0.0;
    bool run = i < a.s.n && (!useTrialBox || ctl.volValid);
    if (run) {
        DevCtx c;
        c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = a.s.n; c.sqmaxcut = a.t.sqmaxcut;
        const double* bx = useTrialBox ? ctl.trialBox : a.s.box;
        double3 box = mk(bx[0], bx[1], bx[2]);
        const Grid& g = a.g;
        PView v = viewAt(a.s, i);
        Con con = makeCon(c, i, a.s.mol[i]);
        for (int q = 0; q < 4; ++q) {
            int j = con.idx[q];
            if (j >= 0 && j < i) {
                unsigned bb; double dd;
                sum += pairEnergy(c, v, viewAt(a.s, j), con, box, &bb, &dd);
            }
        }
        int cell = a.cellOf[i];
        int cx = cell % g.nc[0], cy = (cell / g.nc[0]) % g.nc[1], cz = cell / (g.nc[0] * g.nc[1]);
        int offx[3], offy[3], offz[3];
        int nx = neighbourOffsets(g.nc[0], offx), ny = neighbourOffsets(g.nc[1], offy), nz = neighbourOffsets(g.nc[2], offz);
        for (int qz = 0; qz < nz; ++qz)
            for (int qy = 0; qy < ny; ++qy)
                for (int qx = 0; qx < nx; ++qx) {
                    int x = (cx + offx[qx] + g.nc[0]) % g.nc[0];
                    int y = (cy + offy[qy] + g.nc[1]) % g.nc[1];
                    int z = (cz + offz[qz] + g.nc[2]) % g.nc[2];
                    int c2 = (z * g.nc[1] + y) * g.nc[0] + x;
                    int s2 = a.cellStart[c2], n2 = a.cellCount[c2];
                    for (int k = 0; k < n2; ++k) {
                        int j = a.cellIdx[s2 + k];
                        if (j >= i || j == con.idx[0] || j == con.idx[1] || j == con.idx[2] || j == con.idx[3]) continue;
                        unsigned bb; double dd;
                        sum += pairEnergy(c, v, viewAt(a.s, j), con, box, &bb, &dd);
                    }
                }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < kTotThreads / 32; ++q) s += ws[q];
        a.partial[blockIdx.x] = s;
    }
}

__device__ double sumPartials(const double* p, int n) {
    double s = 0.0;
    for (int k = 0; k < n; ++k) s += p[k];
    return s;
}

// MoveCreator::pressureMove, ptype 1 (movecreator.cpp:390-421), decided on the device.
__global__ void kVolumeAccept(SweepArgs a, int nblocks) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Control& c = *a.ctl;
    if (!c.volValid) {
        atomicAdd(&a.counters[C_VOL_CONSTR], 1ull);
        atomicAdd(&a.counters[C_REJ_V], 1ull);
        return;
    }
    double eNew = sumPartials(a.partial, nblocks);
    double pvol = a.s.box[0] * a.s.box[1] * a.s.box[2];
    double pvoln = c.trialBox[0] * c.trialBox[1] * c.trialBox[2];
    double enermove = a.press * (pvoln - pvol) - (double)a.s.n * a.temper * log(pvoln / pvol);
    enermove += eNew;
    Stream r(a.seed, 0xFFFFFFF1u, (uint32_t)c.sweep, (uint32_t)(c.sweep >> 32));
    double u = r.next();
    double energy = c.energy;
    bool accept = (enermove <= energy) || (exp(-1.0 * (enermove - energy) / a.temper) > u);
    if (accept) {
        for (int d = 0; d < 3; ++d) a.s.box[d] = c.trialBox[d];
        c.energy = eNew;
        atomicAdd(&a.counters[C_ACC_V], 1ull);
    } else {
        atomicAdd(&a.counters[C_REJ_V], 1ull);
    }
}

__global__ void kSetEnergy(SweepArgs a, int nblocks) {
    if (threadIdx.x == 0 && blockIdx.x == 0) a.ctl->energy = sumPartials(a.partial, nblocks);
}

__global__ void kCheckEnergy(SweepArgs a, int nblocks) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double e = sumPartials(a.partial, nblocks);
    Control& c = *a.ctl;
    c.energyCheck = e;
    double d = fabs(c.energy - e);
    if (d > c.maxDrift) c.maxDrift = d;
}

}  // namespace

struct SweepEngine {
    Grid g{};
    Control* ctl = nullptr;
    int *cellStart = nullptr, *cellCount = nullptr, *cellCursor = nullptr, *cellIdx = nullptr, *cellOf = nullptr;
    double* cellDE = nullptr;
    double* partial = nullptr;
    unsigned long long* counters = nullptr;
    int* err = nullptr;
    int ncellsAlloc = 0;
    int nTotBlocks = 0;
    std::vector<void*> allocs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evP0 = nullptr, evP1 = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    SweepArgs graphArgs{};
    long graphBlock = 0, graphLaunches = 0, graphPhaseLaunches = 0;
    bool energyKnown = false;
    uint64_t seed = 0;
    long launches = 0;
};

static int engineAlloc(SweepEngine* e, void** p, size_t bytes) {
    cudaError_t r = cudaMalloc(p, bytes ? bytes : 16);
    if (r != cudaSuccess) return cudaFail(r, "cudaMalloc (sweep)");
    e->allocs.push_back(*p);
    return SC_OK;
}

// Cell grid for a box: cells at least maxcut*(1+margin) wide, an even count per dimension
// (or 1 / 2), so that the 2x2x2 colouring keeps same-colour cells apart.
static Grid makeGrid(const double* box, double maxcut, double margin) {
    Grid g{};
    g.maxcut = maxcut;
    for (int d = 0; d < 3; ++d) {
        int nc = (int)std::floor(box[d] / (maxcut * (1.0 + margin)));
        if (nc < 1) nc = 1;
        if (nc >= 3 && (nc & 1)) nc -= 1;
        g.nc[d] = nc;
        g.p[d] = nc >= 2 ? 2 : 1;
    }
    g.ncells = g.nc[0] * g.nc[1] * g.nc[2];
    g.nactive = (g.nc[0] / g.p[0]) * (g.nc[1] / g.p[1]) * (g.nc[2] / g.p[2]);
    g.ncolours = g.p[0] * g.p[1] * g.p[2];
    return g;
}

void destroyEngine(Context* c) {
    SweepEngine* e = c->engine;
    if (!e) return;
    cudaSetDevice(c->device);
    for (void* p : e->allocs) cudaFree(p);
    for (cudaEvent_t ev : {e->ev0, e->ev1, e->evP0, e->evP1})
        if (ev) cudaEventDestroy(ev);
    if (e->graphExec) cudaGraphExecDestroy(e->graphExec);
    delete e;
    c->engine = nullptr;
}

static int ensureGrid(Context* c, SweepEngine* e, const double* box, double margin) {
    Grid g = makeGrid(box, c->topo.maxcut, margin);
    if (g.ncells > e->ncellsAlloc) {
        for (void** p : {(void**)&e->cellStart, (void**)&e->cellCount, (void**)&e->cellCursor, (void**)&e->cellDE}) {
            if (*p) {
                cudaFree(*p);
                e->allocs.erase(std::find(e->allocs.begin(), e->allocs.end(), *p));
                *p = nullptr;
            }
        }
        int n = g.ncells;
        int rc;
        if ((rc = engineAlloc(e, (void**)&e->cellStart, sizeof(int) * n))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->cellCount, sizeof(int) * n))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->cellCursor, sizeof(int) * n))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->cellDE, sizeof(double) * n))) return rc;
        e->ncellsAlloc = n;
    }
    e->g = g;
    return SC_OK;
}

static SweepArgs makeArgs(Context* c, SweepEngine* e, const sc_run_params& p) {
    SweepArgs a;
    std::memset(&a, 0, sizeof a);
    a.s = c->d;
    a.t = c->tables;
    a.g = e->g;
    a.ctl = e->ctl;
    a.cellStart = e->cellStart; a.cellCount = e->cellCount; a.cellCursor = e->cellCursor;
    a.cellIdx = e->cellIdx; a.cellOf = e->cellOf; a.cellDE = e->cellDE; a.partial = e->partial;
    a.counters = e->counters; a.err = e->err;
    a.seed = p.seed;
    a.temper = p.temper;
    a.press = p.press;
    a.rotAngle = p.rot_angle;
    a.edgeMx = p.edge_mx;
    for (size_t k = 0; k < c->usedTypes.size() && k < (size_t)MAX_DEV_TYPES; ++k) {
        int t = c->usedTypes[k];
        // per-type displacement (sim.h:368-373); the run's transmx replaces the options value
        double base = c->opts.transmx;
        double perType = c->opts.trans_type[t];
        a.trans[k] = (base > 0 && perType != base) ? perType * (p.transmx / base) : p.transmx;
        a.geo[k] = c->topo.ia[t][t].geotype[0];
    }
    return a;
}

// Cell list for the current positions and control block.
static cudaError_t launchCells(const SweepArgs& a, cudaStream_t st, long& launches) {
    int n = a.s.n;
    cudaError_t r = cudaMemsetAsync(a.cellCount, 0, sizeof(int) * a.g.ncells, st);
    if (r != cudaSuccess) return r;
    kAssign<<<(n + 255) / 256, 256, 0, st>>>(a);
    kScan<<<1, 1024, 0, st>>>(a);
    kScatter<<<(n + 255) / 256, 256, 0, st>>>(a);
    kSortCells<<<(a.g.ncells + 127) / 128, 128, 0, st>>>(a);
    launches += 4;
    return cudaGetLastError();
}

int runSweeps(Context* c, const sc_run_params& p, sc_run_stats& st) {
    std::memset(&st, 0, sizeof st);
    if (p.nsweeps < 0) return fail(SC_ERR_ARG, "nsweeps must be >= 0");
    if (!(p.temper > 0)) return fail(SC_ERR_ARG, "temper must be positive");
    if (p.ptype != 0 && p.ptype != 1) return fail(SC_ERR_UNSUPPORTED, "only ptype 1 (isotropic) volume moves run on the GPU");
    int rc = c->ensureDevice();
    if (rc) return rc;
    if (c->d.n == 0) return SC_OK;
    int n = c->d.n;
    SweepEngine* e = c->engine;
    if (!e) {
        e = new SweepEngine();
        c->engine = e;
        if ((rc = engineAlloc(e, (void**)&e->ctl, sizeof(Control)))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->cellIdx, sizeof(int) * n))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->cellOf, sizeof(int) * n))) return rc;
        e->nTotBlocks = (n + kTotThreads - 1) / kTotThreads;
        if ((rc = engineAlloc(e, (void**)&e->partial, sizeof(double) * e->nTotBlocks))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->counters, sizeof(unsigned long long) * C_COUNT))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->err, sizeof(int)))) return rc;
        cudaEventCreate(&e->ev0);
        cudaEventCreate(&e->ev1);
        cudaEventCreate(&e->evP0);
        cudaEventCreate(&e->evP1);
        Control z;
        std::memset(&z, 0, sizeof z);
        cudaMemcpy(e->ctl, &z, sizeof z, cudaMemcpyHostToDevice);
    }
    if (e->seed != p.seed) {
        // a new seed restarts the sweep counter of the Philox streams
        unsigned long long zero = 0;
        cudaMemcpy(&e->ctl->sweep, &zero, sizeof zero, cudaMemcpyHostToDevice);
        e->seed = p.seed;
    }
    cudaStream_t s = c->stream;
    cudaMemsetAsync(e->counters, 0, sizeof(unsigned long long) * C_COUNT, s);
    cudaMemsetAsync(e->err, 0, sizeof(int), s);
    cudaMemsetAsync(&e->ctl->maxDrift, 0, sizeof(double), s);
    double box[3];
    cudaMemcpyAsync(box, c->d.box, sizeof box, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const bool npt = p.ptype == 1 && p.volume_every > 0;
    const double margin = npt ? 0.03 : 1e-9;
    if ((rc = ensureGrid(c, e, box, margin))) return rc;
    SweepArgs a = makeArgs(c, e, p);
    long launches = 0;
    cudaError_t r;
    // exact starting energy (Updater::simulate calls initEM + allToAll, updater.cpp:128-131)
    if (!e->energyKnown || c->hostNewer) {
        kBeginSweep<<<1, 32, 0, s>>>(a, 0);
        if ((r = launchCells(a, s, launches)) != cudaSuccess) return cudaFail(r, "cell list");
        kTotalEnergy<<<e->nTotBlocks, kTotThreads, 0, s>>>(a, 0);
        kSetEnergy<<<1, 32, 0, s>>>(a, e->nTotBlocks);
        e->energyKnown = true;
    }
    cudaEventRecord(e->ev0, s);
    const long chunk = 48;
    double phaseMs = 0.0;
    long phaseLaunches = 0;
    // one sweep: control block, cell list, the colour phases, energy bookkeeping, volume move
    auto launchOne = [&](bool volDue, bool timing) -> cudaError_t {
        kBeginSweep<<<1, 32, 0, s>>>(a, volDue ? 1 : 0);
        cudaError_t r2 = launchCells(a, s, launches);
        if (r2 != cudaSuccess) return r2;
        if (timing) cudaEventRecord(e->evP0, s);
        for (int ph = 0; ph < a.g.ncolours; ++ph) kColour<<<a.g.nactive, kMoveThreads, 0, s>>>(a, ph);
        if (timing) {
            cudaEventRecord(e->evP1, s);
            cudaEventSynchronize(e->evP1);
            float pms = 0;
            cudaEventElapsedTime(&pms, e->evP0, e->evP1);
            phaseMs += pms;
        }
        phaseLaunches += a.g.ncolours;
        kEndSweep<<<1, 256, 0, s>>>(a);
        launches += 2 + a.g.ncolours;
        if (volDue) {
            kTotalEnergy<<<e->nTotBlocks, kTotThreads, 0, s>>>(a, 1);
            kVolumeAccept<<<1, 32, 0, s>>>(a, e->nTotBlocks);
            launches += 2;
        }
        return cudaGetLastError();
    };
    // Blocks of G sweeps are captured once into a CUDA graph and replayed: the kernels
    // read everything that changes from sweep to sweep (sweep index, grid offset, colour
    // order, box, energy) from the device control block.
    const int ve = npt ? p.volume_every : 1;
    const long G = (long)ve * std::max(1, (8 + ve - 1) / ve);
    const bool useGraph = !p.time_phases;
    long nextCheck = p.check_every > 0 ? p.check_every : -1;
    long nextRegrid = npt ? chunk : -1;
    long sw = 0;
    while (sw < p.nsweeps) {
        long left = p.nsweeps - sw;
        if (useGraph && left >= G && sw % G == 0) {
            if (!e->graphExec || std::memcmp(&e->graphArgs, &a, sizeof a) != 0 || e->graphBlock != G) {
                if (e->graphExec) { cudaGraphExecDestroy(e->graphExec); e->graphExec = nullptr; }
                cudaGraph_t graph;
                long before = launches, beforeP = phaseLaunches;
                if ((r = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cudaFail(r, "graph capture");
                for (long k = 0; k < G; ++k) {
                    cudaError_t r2 = launchOne(npt && ((k + 1) % ve == 0), false);
                    if (r2 != cudaSuccess) { cudaStreamEndCapture(s, &graph); return cudaFail(r2, "graph capture launch"); }
                }
                if ((r = cudaStreamEndCapture(s, &graph)) != cudaSuccess) return cudaFail(r, "graph capture end");
                r = cudaGraphInstantiate(&e->graphExec, graph, 0);
                cudaGraphDestroy(graph);
                if (r != cudaSuccess) return cudaFail(r, "graph instantiate");
                e->graphLaunches = launches - before;
                e->graphPhaseLaunches = phaseLaunches - beforeP;
                launches = before;
                phaseLaunches = beforeP;
                e->graphArgs = a;
                e->graphBlock = G;
            }
            if ((r = cudaGraphLaunch(e->graphExec, s)) != cudaSuccess) return cudaFail(r, "graph launch");
            launches += e->graphLaunches;
            phaseLaunches += e->graphPhaseLaunches;
            sw += G;
        } else {
            if ((r = launchOne(npt && ((sw + 1) % ve == 0), p.time_phases != 0)) != cudaSuccess) return cudaFail(r, "sweep launch");
            sw += 1;
        }
        if (nextCheck > 0 && sw >= nextCheck) {
            // the cell list (box fractions) stays valid after an accepted volume move
            kTotalEnergy<<<e->nTotBlocks, kTotThreads, 0, s>>>(a, 0);
            kCheckEnergy<<<1, 32, 0, s>>>(a, e->nTotBlocks);
            launches += 2;
            while (nextCheck <= sw) nextCheck += p.check_every;
        }
        if (nextRegrid > 0 && sw >= nextRegrid && sw < p.nsweeps) {
            // the box changed on the device: re-derive the cell grid when needed
            while (nextRegrid <= sw) nextRegrid += chunk;
            cudaMemcpyAsync(box, c->d.box, sizeof box, cudaMemcpyDeviceToHost, s);
            if ((r = cudaStreamSynchronize(s)) != cudaSuccess) return cudaFail(r, "sweep");
            Grid ng = makeGrid(box, c->topo.maxcut, margin);
            if (ng.nc[0] != a.g.nc[0] || ng.nc[1] != a.g.nc[1] || ng.nc[2] != a.g.nc[2]) {
                if ((rc = ensureGrid(c, e, box, margin))) return rc;
                a = makeArgs(c, e, p);
            }
        }
        if ((r = cudaGetLastError()) != cudaSuccess) return cudaFail(r, "sweep launch");
    }
    cudaEventRecord(e->ev1, s);
    if ((r = cudaStreamSynchronize(s)) != cudaSuccess) return cudaFail(r, "sweep");
    float ms = 0;
    cudaEventElapsedTime(&ms, e->ev0, e->ev1);
    unsigned long long ctr[C_COUNT];
    Control hc;
    int err = 0;
    cudaMemcpy(ctr, e->counters, sizeof ctr, cudaMemcpyDeviceToHost);
    cudaMemcpy(&hc, e->ctl, sizeof hc, cudaMemcpyDeviceToHost);
    cudaMemcpy(&err, e->err, sizeof err, cudaMemcpyDeviceToHost);
    c->devNewer = true;
    st.sweeps = p.nsweeps;
    st.moves = (long)ctr[C_MOVES];
    st.acc_trans = (long)ctr[C_ACC_T]; st.rej_trans = (long)ctr[C_REJ_T];
    st.acc_rot = (long)ctr[C_ACC_R]; st.rej_rot = (long)ctr[C_REJ_R];
    st.acc_vol = (long)ctr[C_ACC_V]; st.rej_vol = (long)ctr[C_REJ_V]; st.vol_constrained = (long)ctr[C_VOL_CONSTR];
    st.pairs_tested = (long)ctr[C_TESTED];
    st.pairs_evaluated = (long)ctr[C_EVAL];
    st.energy = hc.energy;
    st.energy_check = hc.energyCheck;
    st.max_drift = hc.maxDrift;
    st.seconds = ms * 1e-3;
    st.phase_seconds = phaseMs * 1e-3;
    st.phase_launches = phaseLaunches;
    st.launches = launches;
    c->lastLaunches = launches;
    if (err & E_CELL_OVERFLOW) return fail(SC_ERR_DEVICE, "a cell holds more than 256 particles (density too high for the cell list)");
    if (err & E_PARTNER_FAR) return fail(SC_ERR_DEVICE, "a bonded partner lies beyond the neighbouring cells (bond longer than maxcut)");
    return SC_OK;
}

}  // namespace scg
