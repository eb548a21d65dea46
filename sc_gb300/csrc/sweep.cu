// sweep.cu -- the on-device Metropolis move loop (Updater::simulate, scOOP/mc/updater.cpp:45-389).
//
// One sweep = N attempted single-particle moves, run as a checkerboard over a cell
// list so that moves in different cells proceed concurrently without changing the
// stationary distribution:
//   * cells are at least maxcut/s wide (maxcut = sqrt(sqmaxcut), the PairE prefilter
//     range; s = stencil reach), so every particle that can interact with a particle of
//     a cell lies within s cells of it;
//   * each sweep shifts the grid by a random offset, rebuilds the cell list (counting
//     sort), and visits the (s+1)^3 colour classes in random order; two cells of one
//     colour are s+1 cells apart, so their moves are independent;
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
// One CTA owns one active cell.  The candidate partners (the cell and its stencil) are
// staged in shared memory once per launch, positions as FP32 box fractions.  For each
// move, warp 0 builds the proposal (one lane per rotated vector), then three stages
// narrow the work that needs FP64:
//   A  FP32 minimum-image distance of every candidate against the old / new position,
//      with a margin that covers FP32 rounding: a candidate that fails is beyond the
//      FP64 prefilter for certain;
//   B  the FP64 prefilter of PairE (bit-exact) and an FP32 closest segment /
//      point-segment distance: beyond the repulsive and attractive cutoffs (plus a
//      margin) the reference's pair energy is exactly 0, so the pair is dropped;
//   C  the full FP64 PairE of the survivors, one pair per thread.
// Survivors are compacted with deterministic block scans, and the old and new energies
// are summed in a fixed order, so runs are bit-reproducible.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pair_energy.cuh"
#include "philox.cuh"
#include "sc_context.h"
#include "surrogate.cuh"
#include "wanglandau.h"

namespace scg {

namespace {

constexpr int kMoveThreads = 128;
constexpr int kWarps = kMoveThreads / 32;
constexpr int kCellCap = 256;        // particles of a cell staged in shared memory (larger cells: read from the cell list)
constexpr int kNbCap = 343;          // stencil cells, (2*3+1)^3
constexpr int kCandCap = 1024;       // candidates staged in shared memory at a time
constexpr int kQueueCap = 2048;      // pair queue entries (old + new of a full window)
constexpr int kChunk = 512;          // candidates per stage-A round
constexpr int kMaxColours = 64;
constexpr size_t kDynSmem = (size_t)kCandCap * (sizeof(float4) + sizeof(int));
constexpr size_t kDynSmemColour = kDynSmem + (size_t)kCandCap * sizeof(float4);            // + FP32 axes
constexpr size_t kDynSmemSurrogate = kDynSmem + (size_t)kCandCap * 2 * sizeof(float4);   // + FP32 axes, patches

enum Ctr { C_ACC_T, C_REJ_T, C_ACC_R, C_REJ_R, C_ACC_V, C_REJ_V, C_VOL_CONSTR, C_TESTED, C_EVAL, C_CELL_REJ, C_MOVES,
           C_SCREENED, C_S1_REJ, C_S2_TRIED, C_S2_REJ, C_ACC_CH, C_REJ_CH, C_CH_CONSTR, C_ACC_SW, C_REJ_SW, C_COUNT };
enum ErrBit { E_PARTNER_FAR = 2, E_FLOW_WAIT = 4, E_GC_FULL = 8 };
constexpr int kMaxChainTypes = 8;                         // chain molecule types with their own step
constexpr int kTypeCtrChain = 4 * MAX_DEV_TYPES;
constexpr int kTypeCtrCount = kTypeCtrChain + 4 * kMaxChainTypes;

struct Grid {
    int nc[3];
    int p[3];         // colours per dimension (period of the colouring)
    int s[3];         // stencil reach per dimension
    int ncells;
    int nactive;      // cells per colour
    int ncolours;
    double maxcut;
};

// Per-sweep control block, device resident (so that blocks of sweeps replay as a graph).
struct Control {
    unsigned long long sweep;
    double shift[3];      // grid offset, box fractions
    int perm[kMaxColours];
    double psch;          // volume move: edge change
    int volValid;         // trial box keeps cells >= maxcut/s
    int pad_;
    double trialBox[3];
    double pvTerm;        // volume move: P dV - N T ln(V'/V) of the proposal (per ptype)
    double energy;        // running total energy
    double energyCheck;   // last exact total energy
    double maxDrift;
    double daErr2, daErrSum;   // sums of (dE - dEs)^2 and dE - dEs over moves reaching the exact stage
    unsigned epoch;       // sweeps begun, never reset (stamps of the dataflow sweep's cells)
    int ticket;           // next cell of the dataflow sweep
};

struct GcDev;   // grand-canonical species and their record (kGrandCanon)

// What Particle::init (scOOP/structures/particle.cpp:3-79) reads of a particle type.
struct TypeInit {
    int geo;                             // geotype[0]
    int pad_;
    double pcos0, psin0, pcos2, psin2;   // pcoshalfi / psinhalfi of patches 0 and 2
    double csec, ssec;                   // csecpatchrot[0], ssecpatchrot[0]
    double chcos, chsin;                 // chiral_cos[0], chiral_sin[0]
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
    float4* cellPosF;     // wrapped box fractions of cellIdx, FP32
    float4* cellDirF;     // FP32 axis of cellIdx (stage B's screen, the surrogate's inputs)
    float4* cellPatF;     // FP32 first patch direction (written only when a surrogate is attached)
    int* cellOf;
    double* cellDE;
    unsigned* cellDone;   // dataflow sweep: epoch of the sweep in which the cell finished
    double* partial;      // per-cell energy sums
    unsigned long long* counters;
    int* err;
    uint64_t seed;
    double temper, press;
    double rotAngle;
    double edgeMx;
    double trans[MAX_DEV_TYPES];
    int geo[MAX_DEV_TYPES];
    const MlpPacked* mlp;   // delayed acceptance: the surrogate's weights (nullptr: plain moves)
    int pairMoves;          // paired passes in the move kernel (two moves per stage C)
    float rcutS;            // its range (FP32 segment distance)
    // chain moves (records of the chain grid; see kChainColour)
    double* energyAcc;      // where kEndSweep adds the sweep's energy change (nullptr: ctl->energy)
    const int2* chains;     // first particle, size of each chain
    int nChains;
    int* chainCellStart;
    int* chainCellCount;
    int* chainCellIdx;
    int* slotOf;            // chain grid: slot of each particle in cellIdx (written by kSortCells)
    double chainMx;         // chain displacement length
    double chainAngle;      // chain rotation angle bound
    double chainFrac;       // chain move attempts per chain per sweep
    double chainR;          // bound on |particle - chain centre| (real space) the grid was sized for
    double volW[MAX_DEV_TYPES];   // Ia_param volume of each type (clusterCM weights)
    int ptype;              // pressure coupling of volume moves (movecreator.cpp:349-546)
    double boxMinChain[3];  // smallest box edges the chain grid allows (0: no chain phase)
    WlDev* wl;              // Wang-Landau bias (nullptr: none; only the particle grid's records)
    int flowSpin;           // dataflow sweep: polls of one wait before the CTA gives up
    // per-type acceptance of the run (the reference's Disp counters, statistics.h:53-66):
    // [4 t + 0..3] displacement acc / rej, rotation acc / rej of compact type t; then
    // [kTypeCtrChain + 4 m + 0..3] chain displacement acc / rej, rotation acc / rej of molecule type m
    unsigned long long* typeCtr;
    double chainMxType[kMaxChainTypes];   // chain displacement length per molecule type
    double coneAngle;       // options coneAngle (radians): rotations about axes in a cone around the
                            // particle axis (MoveCreator::partAxialRotate); 0: about random axes
    GcDev* gc;              // grand-canonical moves of the run (nullptr: none); kGrandCanon writes
                            // the particle count s.n of these records
    const TypeInit* tinit;  // Particle::init parameters per compact type
    const int4* swTab;      // type switching (nullptr: none): per molecule type and position
                            // (MAXCHL each) compact type, compact switch type (-1), int delta_mu
    double switchRate;      // switch attempts per particle slot of a cell per sweep
};

// One decided single-particle move of compact type `type` in the per-type counters.
__device__ __forceinline__ void countMove(const SweepArgs& a, int type, bool displace, bool accept) {
    if (a.typeCtr && type >= 0 && type < MAX_DEV_TYPES)
        atomicAdd(&a.typeCtr[4 * type + (displace ? 0 : 2) + (accept ? 0 : 1)], 1ull);
}

__device__ __forceinline__ int wrapCell(double x, double shift, int nc) {
    double f = x - floor(x);
    f += shift;
    if (f >= 1.0) f -= 1.0;
    int c = (int)(f * nc);
    return c >= nc ? nc - 1 : (c < 0 ? 0 : c);
}


// Distinct cells of the stencil along one dimension: -s..s, or every cell when the grid
// is narrower than the stencil.
__device__ __forceinline__ int axisCount(int nc, int s) { return nc <= 2 * s ? nc : 2 * s + 1; }
__device__ __forceinline__ int axisCell(int c, int q, int nc, int s) {
    return nc <= 2 * s ? q : (c + q - s + nc) % nc;
}

// Every kernel below serves a batch of independent systems: blockIdx.y selects the
// system, whose arguments live in device memory (so that replica exchange can change a
// system's temperature between launches of a captured graph).
__global__ void kBeginSweep(const SweepArgs* __restrict__ A, int volumeDue) {
    const SweepArgs& a = A[blockIdx.y];
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Control& c = *a.ctl;
    c.epoch += 1;
    c.ticket = 0;
    Stream r(a.seed, 0xFFFFFFF0u, (uint32_t)c.sweep, (uint32_t)(c.sweep >> 32));
    for (int d = 0; d < 3; ++d) c.shift[d] = r.next() / a.g.nc[d];
    int n = a.g.ncolours;
    for (int k = 0; k < n; ++k) c.perm[k] = k;
    for (int k = n - 1; k > 0; --k) {      // Fisher-Yates
        int j = (int)(r.next() * (k + 1));
        if (j > k) j = k;
        int tmp = c.perm[k]; c.perm[k] = c.perm[j]; c.perm[j] = tmp;
    }
    if (a.wl && a.wl->useContacts) {
        // Wang-Landau order 7: the cells whose particles can come within the contact distance
        // of particle 0 wherever it is in its cell (no move leaves its cell): offsets below
        // sqrt(WL_CONTACTS) / width + 1 along each axis, for the box of this sweep
        for (int d = 0; d < 3; ++d) a.wl->reach[d] = (int)(sqrt(kWlContacts) * a.g.nc[d] / a.s.box[d]) + 1;
    }
    c.volValid = 0;
    if (volumeDue) {
        // MoveCreator::pressureMove (movecreator.cpp:330-546): the box proposal and the
        // enthalpy term P dV - N T ln(V'/V) of each pressure coupling
        const double* b = a.s.box;
        double* tb = c.trialBox;
        for (int d = 0; d < 3; ++d) tb[d] = b[d];
        const double NT = (double)a.s.n * a.temper;
        double pv = 0.0;
        switch (a.ptype) {
        case 0: {           // one edge, chosen at random
            double rs = r.next();
            int side = rs < 1.0 / 3.0 ? 0 : (rs < 2.0 / 3.0 ? 1 : 2);
            double area = side == 0 ? b[1] * b[2] : (side == 1 ? b[0] * b[2] : b[0] * b[1]);
            tb[side] += a.edgeMx * (r.next() - 0.5);
            pv = a.press * area * (tb[side] - b[side]) - NT * log(tb[side] / b[side]);
            break;
        }
        case 2: {           // x and y together, z constant
            c.psch = a.edgeMx * (r.next() - 0.5);
            double pvol = b[0] * b[1];
            tb[0] += c.psch; tb[1] += c.psch;
            double pvoln = tb[0] * tb[1];
            pv = a.press * b[2] * (pvoln - pvol) - NT * log(pvoln / pvol);
            break;
        }
        case 3: {           // x and y together, z keeps the volume
            c.psch = a.edgeMx * (r.next() - 0.5);
            double pvol = b[0] * b[1] * b[2];
            tb[0] += c.psch; tb[1] += c.psch;
            tb[2] = pvol / tb[0] / tb[1];
            pv = 0.0;
            break;
        }
        case 4: {           // x or y (the reference's test "if (ran2() - 0.5)" is true unless
                            // the draw is exactly 0.5, so it changes x; kept as it is)
            double pvol = b[0] * b[1];
            if (r.next() - 0.5 != 0.0) tb[0] += a.edgeMx * (r.next() - 0.5);
            else tb[1] += a.edgeMx * (r.next() - 0.5);
            double pvoln = tb[0] * tb[1];
            pv = a.press * b[2] * (pvoln - pvol) - NT * log(pvoln / pvol);
            break;
        }
        case 5: {           // y only
            double pvol = b[1];
            tb[1] += a.edgeMx * (r.next() - 0.5);
            pv = a.press * b[2] * b[0] * (tb[1] - pvol) - NT * log(tb[1] / pvol);
            break;
        }
        default: {          // 1: isotropic
            c.psch = a.edgeMx * (r.next() - 0.5);
            double pvol = b[0] * b[1] * b[2];
            for (int d = 0; d < 3; ++d) tb[d] += c.psch;
            double pvoln = tb[0] * tb[1] * tb[2];
            pv = a.press * (pvoln - pvol) - NT * log(pvoln / pvol);
            break;
        }
        }
        c.pvTerm = pv;
        bool ok = true;
        for (int d = 0; d < 3; ++d) {
            if (!(tb[d] > 0.0) || tb[d] / a.g.nc[d] * a.g.s[d] < a.g.maxcut) ok = false;
            if (tb[d] < a.boxMinChain[d]) ok = false;      // the chain grid must stay valid too
        }
        c.volValid = ok ? 1 : 0;
    }
}

__global__ void kZeroCounts(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.g.ncells) a.cellCount[c] = 0;
}

__global__ void kAssign(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
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
    if (a.wl) {             // the cells of the particles that change the order parameters
        if (i == a.wl->part[0]) a.wl->cell[0] = cell;
        if (i == a.wl->part[1]) a.wl->cell[1] = cell;
    }
}

// Exclusive scan of the cell counts, one CTA of kScanThreads per system.  Each thread owns
// kScanPer consecutive cells of a tile (their loads are independent, so a tile costs one
// memory latency), the thread totals are scanned across the CTA, and the carry moves to the
// next tile: a 40,000-cell grid takes five tiles.
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;

__global__ void __launch_bounds__(kScanThreads) kScan(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    __shared__ int warpTot[kScanThreads / 32];
    const int n = a.g.ncells;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int carry = 0;                         // the same in every thread
    for (int base = 0; base < n; base += kScanThreads * kScanPer) {
        const int k0 = base + (int)threadIdx.x * kScanPer;
        int v[kScanPer];
        int sum = 0;
#pragma unroll
        for (int q = 0; q < kScanPer; ++q) v[q] = k0 + q < n ? a.cellCount[k0 + q] : 0;
#pragma unroll
        for (int q = 0; q < kScanPer; ++q) sum += v[q];
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warpTot[w] = incl;
        __syncthreads();
        int woff = 0, tot = 0;
#pragma unroll
        for (int q = 0; q < kScanThreads / 32; ++q) {
            const int t = warpTot[q];
            if (q < w) woff += t;
            tot += t;
        }
        __syncthreads();
        int run = carry + woff + incl - sum;
#pragma unroll
        for (int q = 0; q < kScanPer; ++q) {
            if (k0 + q < n) {
                a.cellStart[k0 + q] = run;
                a.cellCursor[k0 + q] = 0;
            }
            run += v[q];
        }
        carry += tot;
    }
}

__global__ void kScatter(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.s.n) return;
    int cell = a.cellOf[i];
    int slot = a.cellStart[cell] + atomicAdd(&a.cellCursor[cell], 1);
    a.cellIdx[slot] = i;
}

// Orders each cell's particles by index (deterministic lists whatever the atomics did)
// and writes their FP32 wrapped positions in that order.
__global__ void kSortCells(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.g.ncells) return;
    int s = a.cellStart[c], n = a.cellCount[c];
    int* v = a.cellIdx + s;
    for (int i = 1; i < n; ++i) {
        int x = v[i], j = i - 1;
        while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; --j; }
        v[j + 1] = x;
    }
    for (int k = 0; k < n; ++k) {
        double4_32a p = a.s.pos[v[k]];
        a.cellPosF[s + k] = make_float4(frac32(p.x), frac32(p.y), frac32(p.z), (float)p.w);
        if (a.slotOf) a.slotOf[v[k]] = s + k;
        if (a.cellDirF) {
            double4_32a d = a.s.dir[v[k]];
            a.cellDirF[s + k] = make_float4((float)d.x, (float)d.y, (float)d.z, 0.0f);
        }
        if (a.mlp) {
            const PatchSet& ps = a.s.patch[v[k]];
            a.cellPatF[s + k] = make_float4((float)ps.pd[0][0], (float)ps.pd[0][1], (float)ps.pd[0][2], 0.0f);
        }
    }
}

struct Scan {
    int warpTot[kWarps];
    int nbTot[kWarps];
};

// Exclusive scan of v over the block of NT threads; returns the offset and the total.
template <int NT = kMoveThreads>
__device__ __forceinline__ int blockExclusiveScan(int v, int& total, Scan& sh) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (NT == 32) {                 // one warp: no shared memory, no barrier
        total = __shfl_sync(0xffffffffu, incl, 31);
        return incl - v;
    }
    if (lane == 31) sh.warpTot[w] = incl;
    __syncthreads();
    int woff = 0;
    total = 0;
#pragma unroll
    for (int q = 0; q < NT / 32; ++q) {
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
        for (int q = 0; q < kWarps; ++q) { x += sh[q][0]; y += sh[q][1]; }
    }
    __syncthreads();
}

// Fixed-order block sum of four doubles; results valid in thread 0.
__device__ __forceinline__ void blockSum4(double& x0, double& x1, double& x2, double& x3, double (*sh)[4]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x0 += __shfl_down_sync(0xffffffffu, x0, o);
        x1 += __shfl_down_sync(0xffffffffu, x1, o);
        x2 += __shfl_down_sync(0xffffffffu, x2, o);
        x3 += __shfl_down_sync(0xffffffffu, x3, o);
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sh[w][0] = x0; sh[w][1] = x1; sh[w][2] = x2; sh[w][3] = x3; }
    __syncthreads();
    if (threadIdx.x == 0) {
        x0 = x1 = x2 = x3 = 0.0;
        for (int q = 0; q < kWarps; ++q) { x0 += sh[q][0]; x1 += sh[q][1]; x2 += sh[q][2]; x3 += sh[q][3]; }
    }
    __syncthreads();
}

// Stencil of a cell and the flattened candidate list, shared by the move and energy kernels.
struct Stencil {
    int nbCell[kNbCap];
    int nbOff[kNbCap + 1];
    int nNb;
    int nCand;
    int ownOff;         // offset of the cell's own particles in the candidate list
};

// The stencil of cell (cx, cy, cz): its cells and their offsets in the concatenated
// candidate list (cells in stencil order, particles in cell-list order); NT threads.
template <int NT = kMoveThreads>
__device__ void stageStencil(const SweepArgs& a, int cx, int cy, int cz, Stencil& st, Scan& sc) {
    const Grid& g = a.g;
    const int nx = axisCount(g.nc[0], g.s[0]), ny = axisCount(g.nc[1], g.s[1]), nz = axisCount(g.nc[2], g.s[2]);
    const int nn = nx * ny * nz;
    const int own = g.nc[0] <= 2 * g.s[0] ? cx : g.s[0];
    const int ownY = g.nc[1] <= 2 * g.s[1] ? cy : g.s[1];
    const int ownZ = g.nc[2] <= 2 * g.s[2] ? cz : g.s[2];
    const int ownQ = (ownZ * ny + ownY) * nx + own;
    int carry = 0;
    for (int base = 0; base < nn; base += NT) {
        int q = base + threadIdx.x;
        int cnt = 0, cell = 0;
        if (q < nn) {
            int qx = q % nx, qy = (q / nx) % ny, qz = q / (nx * ny);
            int x = axisCell(cx, qx, g.nc[0], g.s[0]);
            int y = axisCell(cy, qy, g.nc[1], g.s[1]);
            int z = axisCell(cz, qz, g.nc[2], g.s[2]);
            cell = (z * g.nc[1] + y) * g.nc[0] + x;
            cnt = a.cellCount[cell];
        }
        int total;
        int off = blockExclusiveScan<NT>(cnt, total, sc);
        if (q < nn) {
            st.nbCell[q] = cell;
            st.nbOff[q] = carry + off;
        }
        carry += total;
    }
    if (threadIdx.x == 0) {
        st.nNb = nn;
        st.nbOff[nn] = carry;
        st.nCand = carry;
    }
    __syncthreads();
    if (threadIdx.x == 0) st.ownOff = st.nbOff[ownQ];
    __syncthreads();
}

// Loads candidates [first, first + count) of the stencil into shared memory (count <=
// kCandCap).  A stencil larger than the buffer is processed in windows of kCandCap.  NT threads.
template <int NT = kMoveThreads>
__device__ void loadCandidates(const SweepArgs& a, const Stencil& st, int first, int count, int* candIdx,
                               float4* candPos, float4* candDir = nullptr, float4* candPat = nullptr) {
    const int nn = st.nNb;
    for (int kk = threadIdx.x; kk < count; kk += NT) {
        int k = first + kk;
        int lo = 0, hi = nn - 1;      // last q with nbOff[q] <= k
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (st.nbOff[mid] <= k) lo = mid; else hi = mid - 1;
        }
        int slot = a.cellStart[st.nbCell[lo]] + (k - st.nbOff[lo]);
        candIdx[kk] = a.cellIdx[slot];
        candPos[kk] = a.cellPosF[slot];
        if (candDir) candDir[kk] = a.cellDirF[slot];
        if (candPat) candPat[kk] = a.cellPatF[slot];
    }
    __syncthreads();
}

// FP32 closest distance^2 of two segments (centres r apart, r = c1 - c2, unit axes u, v,
// half lengths h1, h2): line solution clamped, then alternating clamped minimisation.
// Any feasible (s, t) bounds the true minimum from above and the error of this
// sequence is far below the screening margin.
__device__ __forceinline__ float segDist2f(float3 r, float3 u, float3 v, float h1, float h2) {
    float b = u.x * v.x + u.y * v.y + u.z * v.z;
    float d = u.x * r.x + u.y * r.y + u.z * r.z;
    float e = v.x * r.x + v.y * r.y + v.z * r.z;
    float den = 1.0f - b * b;
    float s = den > 1e-6f ? (b * e - d) / den : 0.0f;
    s = fminf(fmaxf(s, -h1), h1);
    float t = fminf(fmaxf(b * s + e, -h2), h2);
    s = fminf(fmaxf(b * t - d, -h1), h1);
    t = fminf(fmaxf(b * s + e, -h2), h2);
    float x = r.x + s * u.x - t * v.x, y = r.y + s * u.y - t * v.y, z = r.z + s * u.z - t * v.z;
    return x * x + y * y + z * z;
}

__device__ __forceinline__ float pointSegDist2f(float3 rc, float3 u, float h) {
    float c = u.x * rc.x + u.y * rc.y + u.z * rc.z;
    c = fminf(fmaxf(c, -h), h);
    float x = -rc.x + u.x * c, y = -rc.y + u.y * c, z = -rc.z + u.z * c;
    return x * x + y * y + z * z;
}

// True when the pair energy is exactly zero by the screen of PairParam (and the pair is
// not bonded, which the callers exclude).
__device__ __forceinline__ bool screenedOutF(const PairParam& pp, float3 r, float3 u, float3 v) {
    if (pp.screen == 3) return true;
    if (pp.screen == 0) return false;
    float dd;
    if (pp.screen == 1) {
        dd = segDist2f(r, u, v, (float)pp.half_len[0], (float)pp.half_len[1]);
    } else if (pp.scFirst) {
        dd = pointSegDist2f(r, u, (float)pp.scHalf);
    } else {
        dd = pointSegDist2f(make_float3(-r.x, -r.y, -r.z), v, (float)pp.scHalf);
    }
    return dd > (float)pp.screenSq * 1.001f + 1e-3f;
}
__device__ __forceinline__ bool screenedOut(const PairParam& pp, const double3& r_cm, const double3& d1,
                                           const double3& d2) {
    return screenedOutF(pp, make_float3((float)r_cm.x, (float)r_cm.y, (float)r_cm.z),
                        make_float3((float)d1.x, (float)d1.y, (float)d1.z), make_float3((float)d2.x, (float)d2.y, (float)d2.z));
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

// FP32 candidate threshold: (maxcut + margin)^2, the margin covering the FP32 rounding
// of wrapped box fractions times the box.
__device__ __forceinline__ float candThreshold(double sqmaxcut, const double3& box) {
    double bmax = fmax(box.x, fmax(box.y, box.z));
    double r = sqrt(sqmaxcut) + 1e-6 * bmax + 1e-5;
    return (float)(r * r) * 1.0001f;
}

__device__ __forceinline__ float dist2f(float4 a, float3 b, const double3& box) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    dx -= rintf(dx); dy -= rintf(dy); dz -= rintf(dz);
    dx *= (float)box.x; dy *= (float)box.y; dz *= (float)box.z;
    return dx * dx + dy * dy + dz * dz;
}

constexpr int kClassCap = 768;       // stage-C queue entries per pair class

// Pair class of the stage-C queue: 0 patchy SC-SC pairs (evaluated as parallel chains),
// 1 SC-sphere, 2 everything else.  Each class is evaluated by its own warps, so a warp
// follows one functor's branches.
__device__ __forceinline__ int pairClass(const PairParam& pp) {
    return pp.simple ? 0 : (pp.kind >= K_MIX_SCA_SPA ? 1 : 2);
}

// Barrier of warps 0-2 only (warp 3 keeps evaluating other pairs meanwhile).
__device__ __forceinline__ void barWarps012() { asm volatile("bar.sync 1, 96;" ::: "memory"); }

// Stage-C scratch of the parallel-chain evaluation of class-0 pairs, 32 pairs per round.
struct SplitShared {
    double T[4][32][2], S[4][32][2];     // intersections of each patch combination
    double e0[32];
    double atrA[4][32], f0[4][32], f1[4][32], f2[4][32], paral[4][32];
    int na[4][32], nb[4][32], ok[32];
};

// Up to 32 class-0 pairs (entries queue[r0, r0 + 32), get(entry, self, other) resolves one)
// on warps 0-2.  The WCA chain and the two intersection chains of every valid patch
// combination are separate tasks (task t: 0 WCA, 1 + 2c first and 2 + 2c second
// intersection of combination c; warp w takes t = w, w + 3, w + 6), then the two halves of
// the attraction of every combination with two intersections on each side (A on warp
// c mod 3, B on warp c + 1 mod 3), then warp 0 adds them in combination order -- the
// value of scScEnergy, whose loop runs the same chains one after another.  Returns the
// pair energy of entry r0 + lane to the lanes of warp 0.
__device__ __noinline__ void patchyTask(SplitShared& sp, const PairParam& ia, const PView& self, const PView& b,
                                        const double3& r_cm, int t, int lane) {
    if (t == 0) { sp.e0[lane] = patchyWca(ia, self, b, r_cm, &sp.ok[lane]); return; }
    const int cc = (t - 1) >> 1;
    const bool second = (t - 1) & 1;
    if (!comboValid(ia, cc)) {
        if (second) sp.nb[cc][lane] = 0; else sp.na[cc][lane] = 0;
    } else if (second) {
        sp.nb[cc][lane] = comboIntersect2(ia, self, b, r_cm, cc, sp.S[cc][lane]);
    } else {
        sp.na[cc][lane] = comboIntersect1(ia, self, b, r_cm, cc, sp.T[cc][lane]);
    }
}
__device__ __noinline__ void patchyAttr(SplitShared& sp, const PairParam& ia, const PView& self, const PView& b,
                                        const double3& r_cm, int warp, int lane) {
    for (int cc = 0; cc < 4; ++cc) {
        if (!(sp.na[cc][lane] >= 2 && sp.nb[cc][lane] >= 2)) continue;
        if (warp == cc % 3)
            sp.atrA[cc][lane] = comboAttrA(ia, self, b, r_cm, cc, sp.T[cc][lane], sp.S[cc][lane], &sp.f0[cc][lane]);
        if (warp == (cc + 1) % 3)
            comboAttrB(ia, self, b, r_cm, cc, sp.T[cc][lane], sp.S[cc][lane], &sp.f1[cc][lane], &sp.f2[cc][lane],
                       &sp.paral[cc][lane]);
    }
}

template <class Get>
__device__ double patchyRound(SplitShared& sp, const DevCtx& c, const double3& box, const int* queue, int count,
                              int r0, Get get) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool have = r0 + lane < count;
    PView self, b;
    const PairParam* iap = nullptr;
    double3 r_cm = mk(0.0, 0.0, 0.0);
    if (have) {
        get(queue[r0 + lane], self, b);
        iap = &c.params[self.type * c.ntypes + b.type];
        r_cm = imageVec(self.pos, b.pos, box);
        for (int t = warp; t < 9; t += 3) patchyTask(sp, *iap, self, b, r_cm, t, lane);
    }
    barWarps012();
    if (have && sp.ok[lane]) patchyAttr(sp, *iap, self, b, r_cm, warp, lane);
    barWarps012();
    double e = 0.0;
    if (warp == 0 && have) {
        double atr = 0.0;
        if (sp.ok[lane])
            for (int cc = 0; cc < 4; ++cc)
                if (sp.na[cc][lane] >= 2 && sp.nb[cc][lane] >= 2)
                    atr += patchAttractionCombine(sp.atrA[cc][lane], sp.f0[cc][lane], sp.f1[cc][lane], sp.f2[cc][lane],
                                                  sp.paral[cc][lane]);
        e = sp.e0[lane] + atr;
    }
    barWarps012();            // the scratch is reused by the next round
    return e;
}

__device__ __forceinline__ bool partnerInStencil(const SweepArgs& a, const int* nbCell, int nNb, int j) {
    int cj = a.cellOf[j];
    bool near = false;
    for (int w = 0; w < nNb; ++w) near |= (nbCell[w] == cj);
    return near;
}

// One move's proposal.  thrMet / thrStage1: the move is accepted when dE <= 0 or
// dE < thr, thr = -T ln(u) -- the reference's exp(-dE/T) > u (movecreator.h:175-187)
// with the logarithm taken while the proposal is built, off the critical path.
struct Proposal {
    int target, slotR, displace, skip, partners[4], nPartners, type;
    double thrMet, thrStage1;
    double opos[3], odir[3], dirW;      // the target's state the proposal was built from
    double npos[3], ndir[3];
    float3 oldF, newF;
    PatchSet npatch;
};

struct MoveShared {
    int list[kCellCap];
    int queueA[kQueueCap];
    int queueB[3][kClassCap];
    Stencil st;
    Scan scan;
    double red[kWarps][4];
    SplitShared split;
    // surrogate stage: per-warp input rows, WCA32 and sign (+1 new, -1 old) of each row
    float sx[kWarps][16][kFeat];
    float swca[kWarps][16];
    float ssign[kWarps][16];
    float sred[kWarps];
    // proposals: move k in slot k & 3; propFor[slot] is the move the slot holds (-1: none)
    Proposal prop[4];
    int propFor[4];
    int passDone;       // moves a pass decided (1 or 2)
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

// Warp 0 builds the proposal of move m.  Particle::pscRotate (particle.h:182-272): every
// lane forms the rotation matrix, lane k rotates vector k (axis, patch directions, patch
// sides, chiral axes), then patchdir[0] is re-orthogonalised against the new axis as
// partRotate does (movecreator.cpp:1007).
__device__ void buildProposal(const SweepArgs& a, const int* list, const int* nbCell, int nNb, Proposal& P, int cell,
                              int cnt, int m, int cx, int cy, int cz, const double3& box) {
    const Control& ctl = *a.ctl;
    const int lane = threadIdx.x & 31;
    Stream r(a.seed, (uint32_t)cell, (uint32_t)m, (uint32_t)ctl.sweep ^ ((uint32_t)(ctl.sweep >> 32) << 20));
    int slotR = min((int)(r.next() * cnt), cnt - 1);
    int t = list[slotR];
    double4_32a p = a.s.pos[t];
    double4_32a d = a.s.dir[t];
    int type = (int)p.w;
    int geo = a.geo[type];
    bool displace = (r.next() < 0.5) || geo >= SP;
    int skip = 0;
    double npx = p.x, npy = p.y, npz = p.z;
    if (displace) {
        double x, y, z;
        randomUnitSphere(r, x, y, z);
        double mx = a.trans[type];
        x *= mx / box.x; y *= mx / box.y; z *= mx / box.z;
        npx = p.x + x; npy = p.y + y; npz = p.z + z;
        int nx = wrapCell(npx, ctl.shift[0], a.g.nc[0]);
        int ny = wrapCell(npy, ctl.shift[1], a.g.nc[1]);
        int nz = wrapCell(npz, ctl.shift[2], a.g.nc[2]);
        if (nx != cx || ny != cy || nz != cz) skip = 1;     // would leave the cell
        if (lane == 0) { P.ndir[0] = d.x; P.ndir[1] = d.y; P.ndir[2] = d.z; }
    } else {
        double angle = a.rotAngle * r.next();
        double ax, ay, az;
        if (a.coneAngle != 0.0) {
            // MoveCreator::partAxialRotate (movecreator.cpp:1030-1073): the axis is
            // Vector::getRandomUnitConeUniform(dir, coneAngle) (Vector.h:294-308) -- a vector
            // orthogonal to dir (getOrthogonalVector, :256-260) turned about dir by a random angle
            // (getRandomOrthogonalVector, :268-277, Vector::rotate, :138-160), mixed with dir so
            // that the axis' component along dir is uniform in [cos(coneAngle), 1]
            double ox = -d.y, oy = d.x, oz = 0.0;
            if (d.x == 0.0 && d.y == 0.0) { ox = 0.0; oy = 1.0; oz = 0.0; }
            const double cr = cos(r.next() * 2.0 * 3.141592653589793238462643383279);
            const double sr = sqrt(1.0 - cr * cr);
            const double qx = d.x * sr, qy = d.y * sr, qz = d.z * sr;
            const double t2 = cr * qx, t3 = cr * qy, t4 = cr * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz,
                         t8 = -qy * qy, t9 = qy * qz, t10 = -qz * qz;
            const double rx = 2.0 * ((t8 + t10) * ox + (t6 - t4) * oy + (t3 + t7) * oz) + ox;
            const double ry = 2.0 * ((t4 + t6) * ox + (t5 + t10) * oy + (t9 - t2) * oz) + oy;
            const double rz = 2.0 * ((t7 - t3) * ox + (t2 + t9) * oy + (t5 + t8) * oz) + oz;
            const double cosA = cos(a.coneAngle);
            const double mult = r.next() * (1.0 - cosA) + cosA;
            const double dl = 1.0 / sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
            const double ol = 1.0 / sqrt(rx * rx + ry * ry + rz * rz);
            const double side = sqrt(1.0 - mult * mult);
            ax = d.x * dl * mult + side * (rx * ol);
            ay = d.y * dl * mult + side * (ry * ol);
            az = d.z * dl * mult + side * (rz * ol);
        } else {
            randomUnitSphere(r, ax, ay, az);
        }
        bool positive = r.next() < 0.5;
        double vc = cos(angle);
        double vs = positive ? sqrt(1.0 - vc * vc) : -sqrt(1.0 - vc * vc);
        double qw = vc, qx = ax * vs, qy = ay * vs, qz = az * vs;
        double t2 = qw * qx, t3 = qw * qy, t4 = qw * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
               t9 = qy * qz, t10 = -qz * qz;
        double d1 = t8 + t10, d2 = t6 - t4, d3 = t3 + t7, d4 = t4 + t6, d5 = t5 + t10, d6 = t9 - t2, d7 = t7 - t3,
               d8 = t2 + t9, d9 = t5 + t8;
        // lane k: 0 axis, 1-2 patchdir, 3-6 patchsides, 7-8 chdir
        const PatchSet& ps = a.s.patch[t];
        double v[3];
        bool rotate;
        int twoP = isTwoPatch(geo) ? 2 : 1;
        int twoC = (geo == TCHPSC || geo == TCHCPSC) ? 2 : 1;
        if (lane == 0) { v[0] = d.x; v[1] = d.y; v[2] = d.z; rotate = true; }
        else if (lane <= 2) { for (int q = 0; q < 3; ++q) v[q] = ps.pd[lane - 1][q]; rotate = geo != SCN && geo != SCA && (lane - 1) < twoP; }
        else if (lane <= 6) { for (int q = 0; q < 3; ++q) v[q] = ps.ps[lane - 3][q]; rotate = geo != SCN && geo != SCA && ((lane - 3) >> 1) < twoP; }
        else if (lane <= 8) { for (int q = 0; q < 3; ++q) v[q] = ps.ch[lane - 7][q]; rotate = isChiral(geo) && (lane - 7) < twoC; }
        else { v[0] = v[1] = v[2] = 0.0; rotate = false; }
        if (rotate) {
            double nx = 2.0 * (d1 * v[0] + d2 * v[1] + d3 * v[2]) + v[0];
            double ny = 2.0 * (d4 * v[0] + d5 * v[1] + d6 * v[2]) + v[1];
            double nz = 2.0 * (d7 * v[0] + d8 * v[1] + d9 * v[2]) + v[2];
            v[0] = nx; v[1] = ny; v[2] = nz;
        }
        double dx = __shfl_sync(0xffffffffu, v[0], 0), dy = __shfl_sync(0xffffffffu, v[1], 0),
               dz = __shfl_sync(0xffffffffu, v[2], 0);
        if (lane == 1 && a.coneAngle == 0.0) {      // partRotate re-orthogonalises, partAxialRotate does not
            double dp = v[0] * dx + v[1] * dy + v[2] * dz;
            v[0] -= dp * dx; v[1] -= dp * dy; v[2] -= dp * dz;
        }
        if (lane == 0) { P.ndir[0] = v[0]; P.ndir[1] = v[1]; P.ndir[2] = v[2]; }
        else if (lane <= 2) { for (int q = 0; q < 3; ++q) P.npatch.pd[lane - 1][q] = v[q]; }
        else if (lane <= 6) { for (int q = 0; q < 3; ++q) P.npatch.ps[lane - 3][q] = v[q]; }
        else if (lane <= 8) { for (int q = 0; q < 3; ++q) P.npatch.ch[lane - 7][q] = v[q]; }
    }
    if (lane == 0) {
        P.target = t;
        P.slotR = slotR;
        P.displace = displace;
        P.type = type;
        P.opos[0] = p.x; P.opos[1] = p.y; P.opos[2] = p.z;
        P.odir[0] = d.x; P.odir[1] = d.y; P.odir[2] = d.z;
        P.dirW = d.w;
        P.npos[0] = npx; P.npos[1] = npy; P.npos[2] = npz;
        P.oldF = make_float3(frac32(p.x), frac32(p.y), frac32(p.z));
        P.newF = make_float3(frac32(npx), frac32(npy), frac32(npz));
        // bonded partners are evaluated explicitly; they must sit inside the stencil
        DevCtx c;
        c.mols = a.t.mols;
        Con con = makeCon(c, t, a.s.mol[t]);
        int np = 0;
        for (int q = 0; q < 4; ++q) {
            int j = con.idx[q];
            if (j < 0) continue;
            if (!partnerInStencil(a, nbCell, nNb, j)) { atomicOr(a.err, E_PARTNER_FAR); skip = 1; }
            P.partners[np++] = j;
        }
        P.nPartners = np;
        P.skip = skip;
    }
}

__device__ __forceinline__ bool isPartner(const Proposal& P, int j) {
    bool r = false;
    for (int q = 0; q < P.nPartners; ++q) r |= (P.partners[q] == j);
    return r;
}

// The moved particle of proposal P in its old (isNew = false) or new configuration.
__device__ __forceinline__ PView moveView(const DevState& s, const Proposal& P, bool isNew) {
    PView v;
    v.type = P.type;
    v.index = P.target;
    v.molType = 0;
    if (isNew) {
        v.pos = mk(P.npos[0], P.npos[1], P.npos[2]);
        v.dir = mk(P.ndir[0], P.ndir[1], P.ndir[2]);
        v.patch = P.displace ? &s.patch[P.target] : &P.npatch;
    } else {
        v.pos = mk(P.opos[0], P.opos[1], P.opos[2]);
        v.dir = mk(P.odir[0], P.odir[1], P.odir[2]);
        v.patch = &s.patch[P.target];
    }
    return v;
}

// The uniforms of the acceptance tests come from their own Philox stream, so that one
// lane can turn them into thresholds while another warp builds the proposal.
__device__ void acceptThresholds(const SweepArgs& a, Proposal& P, int cell, int m) {
    const Control& ctl = *a.ctl;
    Stream r(a.seed ^ 0xD1B54A32D192ED03ull, (uint32_t)cell, (uint32_t)m,
             (uint32_t)ctl.sweep ^ ((uint32_t)(ctl.sweep >> 32) << 20));
    double u = r.next(), u1 = r.next();
    P.thrMet = -a.temper * log(u);        // +inf for u = 0: always accepted, as exp(.) > 0
    P.thrStage1 = -a.temper * log(u1);
}



// ---- Wang-Landau bias (cells holding the order parameters' particles) -------------------
// The cells that hold particles 0 / 1 (the particles whose moves change the supported order
// parameters) are not moved in their colour phase: kWlCells moves them, one after the other,
// after every other cell of the sweep, so that each of their moves sees the current bins and
// weights, exactly as the reference's sequential loop does for some order of the sweep's moves.
// With order 7 the block of cells within w.reach of particle 0's cell (every cell along an
// axis the block spans whole) joins them: only their particles can change the contact count.
__device__ __forceinline__ bool wlNear(int c, int c0, int nc, int r) {
    if (nc <= 2 * r) return true;
    int d = c > c0 ? c - c0 : c0 - c;
    if (nc - d < d) d = nc - d;
    return d <= r;
}
__device__ __forceinline__ bool wlInBlock(const WlDev& w, const Grid& g, int cell) {
    const int c0 = w.cell[0];
    if (!w.useContacts || c0 < 0 || c0 >= g.ncells) return false;
    return wlNear(cell % g.nc[0], c0 % g.nc[0], g.nc[0], w.reach[0]) &&
           wlNear((cell / g.nc[0]) % g.nc[1], (c0 / g.nc[0]) % g.nc[1], g.nc[1], w.reach[1]) &&
           wlNear(cell / (g.nc[0] * g.nc[1]), c0 / (g.nc[0] * g.nc[1]), g.nc[2], w.reach[2]);
}
__device__ __forceinline__ bool isWlCell(const WlDev& w, const Grid& g, int cell) {
    return cell == w.cell[0] || cell == w.cell[1] || wlInBlock(w, g, cell);
}
// The cells kWlCells moves, in its order: slots 0 .. wlCellSlots - 1, each a cell or -1 (a
// slot with none, or a cell an earlier slot holds).  Without order 7: particle 0's cell, then
// particle 1's; with it: the block around particle 0's cell, then particle 1's cell when the
// block misses it.
__device__ __forceinline__ int wlCellSlots(const WlDev& w, const Grid& g) {
    if (!w.useContacts) return 2;
    return axisCount(g.nc[0], w.reach[0]) * axisCount(g.nc[1], w.reach[1]) * axisCount(g.nc[2], w.reach[2]) + 1;
}
__device__ int wlCellAt(const WlDev& w, const Grid& g, int k) {
    if (!w.useContacts || k == wlCellSlots(w, g) - 1) {
        const int q = w.useContacts ? 1 : k;
        const int cell = w.cell[q];
        if (cell < 0 || cell >= g.ncells || (q == 1 && cell == w.cell[0])) return -1;
        if (w.useContacts && wlInBlock(w, g, cell)) return -1;
        return cell;
    }
    const int c0 = w.cell[0];
    if (c0 < 0 || c0 >= g.ncells) return -1;
    const int nx = axisCount(g.nc[0], w.reach[0]), ny = axisCount(g.nc[1], w.reach[1]);
    const int qx = k % nx, qy = (k / nx) % ny, qz = k / (nx * ny);
    const int x = axisCell(c0 % g.nc[0], qx, g.nc[0], w.reach[0]);
    const int y = axisCell((c0 / g.nc[0]) % g.nc[1], qy, g.nc[1], w.reach[1]);
    const int z = axisCell(c0 / (g.nc[0] * g.nc[1]), qz, g.nc[2], w.reach[2]);
    return (z * g.nc[1] + y) * g.nc[0] + x;
}

// One visit of the current bin (WangLandau::accept / reject, wanglandau.h:262-290): the
// histogram counts it and the weight drops by alpha (implicit in wlWeight).
__device__ __forceinline__ void wlVisit(WlDev& w) {
    atomicAdd((unsigned long long*)&w.tab->hist[wlIndex(w, w.cur)], 1ull);
}

// The bins after proposal P (WangLandau::run for displacements, runRot for rotations,
// wanglandau.h:124-217) and the system centre after it (zDir, :293-299); false when a bin
// leaves the histogram (the move is rejected).
__device__ bool wlProposal(const SweepArgs& a, const WlDev& w, const Proposal& P, const double3& box, long long nw[2],
                           double cmNew[3], long long& contactsNew) {
    const int t = P.target;
    contactsNew = w.contacts;
    for (int d = 0; d < 3; ++d) cmNew[d] = w.syscm[d];
    if (P.displace && w.needCM) {
        const double vol = a.volW[P.type];
        for (int d = 0; d < 3; ++d) cmNew[d] += ((P.npos[d] - P.opos[d]) * vol) / w.sysvol;
    }
    nw[0] = w.cur[0];
    nw[1] = w.cur[1];
    const double bx[3] = {box.x, box.y, box.z};
    for (int k = 0; k < w.dim; ++k) {
        switch (w.wlm[k]) {
        case 1:             // z of particle 0 relative to the centre: every displacement moves the centre
            if (P.displace) nw[k] = wlZOrder(w, k, t == 0 ? P.npos[2] : a.s.pos[0].z, cmNew[2], box.z);
            break;
        case 3:             // z component of particle 0's axis: its rotations
            if (!P.displace && t == 0) nw[k] = wlOrientOrder(w, k, P.ndir[2]);
            break;
        case 4:             // xy distance of particles 0 and 1: their displacements
            if (P.displace && (t == 0 || t == 1)) {
                double p0[3], p1[3];
                const double4_32a q0 = a.s.pos[0], q1 = a.s.pos[1];
                p0[0] = q0.x; p0[1] = q0.y; p0[2] = q0.z;
                p1[0] = q1.x; p1[1] = q1.y; p1[2] = q1.z;
                double* moved = t == 0 ? p0 : p1;
                for (int d = 0; d < 3; ++d) moved[d] = P.npos[d];
                nw[k] = wlDistOrder(w, k, p0, p1, bx);
            }
            break;
        case 7:             // contacts with particle 0 (contParticlesMoveMolecule, wanglandau.h:516-532):
                            // recounted when particle 0 moves, else the moved particle's old and
                            // new contact (only displacements of the counted type change it)
            if (P.displace) {
                if (t == 0) {
                    long long n = 0;
                    for (int i = 1; i < a.s.n; ++i) {
                        const double4_32a q = a.s.pos[i];
                        const double pi[3] = {q.x, q.y, q.z};
                        if ((int)q.w == w.contactType && wlInContact(pi, P.npos, bx)) ++n;
                    }
                    contactsNew = n;
                } else if (P.type == w.contactType) {
                    const double4_32a q0 = a.s.pos[0];
                    const double p0[3] = {q0.x, q0.y, q0.z};
                    contactsNew += (wlInContact(P.npos, p0, bx) ? 1 : 0) - (wlInContact(P.opos, p0, bx) ? 1 : 0);
                }
                nw[k] = wlContactOrder(w, k, contactsNew);
            }
            break;
        default:            // 8, 9: box lengths, changed by volume moves only
            break;
        }
    }
    return wlInRange(w, nw);
}

__device__ __forceinline__ float3 f3(double x, double y, double z) { return make_float3((float)x, (float)y, (float)z); }

// The moved particle as the surrogate sees it (FP32, old and new orientation).
struct MovedF {
    float3 aOld, pOld, aNew, pNew;
    int type;
    float tc;
};

// Surrogate screen of candidate k (shared-memory slot): bit 0 the old, bit 1 the new
// configuration of the moved particle lies within rcutS of it (FP32 segment distance).
__device__ __forceinline__ int surrogateScreen(const SweepArgs& a, const MovedF& mv, float4 cp, float4 cd,
                                               bool displace, float3 oldF, float3 newF, float bx, float by, float bz) {
    const PairParam& pp = a.t.params[mv.type * a.t.ntypes + (int)cp.w];
    if (pp.screen != 1) return 0;
    float h1 = (float)pp.half_len[0], h2 = (float)pp.half_len[1];
    float reach = a.rcutS + h1 + h2;
    float3 ro = pairVecF(oldF, cp, bx, by, bz);
    float3 rn = displace ? pairVecF(newF, cp, bx, by, bz) : ro;
    bool no = dotf(ro, ro) <= reach * reach, nn = dotf(rn, rn) <= reach * reach;
    int flags = 0;
    if (no || nn) {
        float3 aj = make_float3(cd.x, cd.y, cd.z);
        const float rc2 = a.rcutS * a.rcutS;
        float s_, t_;
        float3 w_;
        if (no && segClosestF(ro, mv.aOld, aj, h1, h2, s_, t_, w_) < rc2) flags |= 1;
        if (nn && segClosestF(rn, mv.aNew, aj, h1, h2, s_, t_, w_) < rc2) flags |= 2;
    }
    return flags;
}

// Network rows of queue entries queue[0..n) (slot << 1 | new): warp w takes tiles w, w + 4,
// ...; returns this warp's share of sum(sign * (WCA32 + MLP)), summed in a fixed order.
__device__ __noinline__ float surrogateTiles(const SweepArgs& a, MoveShared& sh, const MovedF& mv, const int* queue, int n,
                                const float4* candPos, const float4* candDir, const float4* candPat, float3 oldF,
                                float3 newF) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float bx = (float)a.s.box[0], by = (float)a.s.box[1], bz = (float)a.s.box[2];
    const int nt = a.t.ntypes;
    float warpSum = 0.0f;
    for (int tile = warp; tile * 16 < n; tile += kWarps) {
        if (lane < 16) {
            int e = tile * 16 + lane;
            float* f = sh.sx[warp][lane];
            float wv = 0.0f, sign = 0.0f;
            if (e < n) {
                int q = queue[e];
                int k = q >> 1;
                bool isNew = q & 1;
                float4 cp = candPos[k], cd = candDir[k], cq = candPat[k];
                int tj = (int)cp.w;
                const PairParam& pp = a.t.params[mv.type * nt + tj];
                float3 r = pairVecF(isNew ? newF : oldF, cp, bx, by, bz);
                float d2 = pairFeatures(r, isNew ? mv.aNew : mv.aOld, isNew ? mv.pNew : mv.pOld, (float)pp.half_len[0],
                                        mv.tc, make_float3(cd.x, cd.y, cd.z), make_float3(cq.x, cq.y, cq.z),
                                        (float)pp.half_len[1], typeCode(tj, nt), f);
                wv = wca32(d2, (float)pp.sigma, (float)pp.epsilon, (float)pp.rcutwcaSq);
                sign = isNew ? 1.0f : -1.0f;
            } else {
                for (int c = 0; c < kFeat; ++c) f[c] = 0.0f;
            }
            sh.swca[warp][lane] = wv;
            sh.ssign[warp][lane] = sign;
        }
        __syncwarp();
        float y0, y1;
        mlpForward16(a.mlp, sh.sx[warp], y0, y1);
        float v = 0.0f;
        if ((lane & 3) == 0) {
            int g = lane >> 2;
            v = sh.ssign[warp][g] * (y0 + sh.swca[warp][g]) + sh.ssign[warp][g + 8] * (y1 + sh.swca[warp][g + 8]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        warpSum += v;
        __syncwarp();
    }
    return warpSum;
}

// The per-warp sums of the surrogate stage, added in a fixed order.
__device__ __forceinline__ float surrogateTotal(MoveShared& sh, float warpSum) {
    if ((threadIdx.x & 31) == 0) sh.sred[threadIdx.x >> 5] = warpSum;
    __syncthreads();
    return ((sh.sred[0] + sh.sred[1]) + sh.sred[2]) + sh.sred[3];
}

// Surrogate energy change of the proposal when the stencil does not fit in shared memory:
// the candidates window by window (the resident case fuses this screen into stage A).
__device__ __noinline__ float surrogateDeltaWindows(const SweepArgs& a, MoveShared& sh, const MovedF& mv,
                                                    int* candIdx, float4* candPos, float4* candDir, float4* candPat,
                                                    int nCand, int t, bool displace, const int (&partners)[4],
                                                    float3 oldF, float3 newF) {
    const int tid = threadIdx.x;
    const float bx = (float)a.s.box[0], by = (float)a.s.box[1], bz = (float)a.s.box[2];
    float warpSum = 0.0f;
    for (int wbase = 0; wbase < nCand; wbase += kCandCap) {
        const int wend = min(wbase + kCandCap, nCand);
        loadCandidates(a, sh.st, wbase, wend - wbase, candIdx, candPos, candDir, candPat);
        int qs = 0;
        for (int r0 = wbase; r0 < wend; r0 += kMoveThreads) {
            int k = r0 + tid - wbase;
            int flags = 0;
            if (r0 + tid < wend) {
                int j = candIdx[k];
                bool partner = (j == partners[0] || j == partners[1] || j == partners[2] || j == partners[3]);
                if (j != t && !partner) flags = surrogateScreen(a, mv, candPos[k], candDir[k], displace, oldF, newF, bx, by, bz);
            }
            int total;
            int off = blockExclusiveScan(__popc(flags), total, sh.scan);
            if (flags & 1) sh.queueA[qs + off++] = k << 1;
            if (flags & 2) sh.queueA[qs + off] = (k << 1) | 1;
            qs += total;
        }
        __syncthreads();
        warpSum += surrogateTiles(a, sh, mv, sh.queueA, qs, candPos, candDir, candPat, oldF, newF);
        __syncthreads();            // queueA and the window are reused
    }
    return surrogateTotal(sh, warpSum);
}

__device__ __forceinline__ void decodeActive(const Grid& g, int colour, int block, int& cx, int& cy, int& cz) {
    int ox = colour % g.p[0], oy = (colour / g.p[0]) % g.p[1], oz = colour / (g.p[0] * g.p[1]);
    int ax = g.nc[0] / g.p[0], ay = g.nc[1] / g.p[1];
    int bx = block % ax, by = (block / ax) % ay, bz = block / (ax * ay);
    cx = ox + g.p[0] * bx; cy = oy + g.p[1] * by; cz = oz + g.p[2] * bz;
}

// No wait: the colour-phase kernels run a cell when its whole phase may run.
struct NoWait {
    __device__ bool operator()() const { return true; }
};

// The moves of cell (cx, cy, cz), by the whole CTA: the move kernel body, run once per CTA
// by the colour-phase kernels (kColour / kColourDense) and once per taken cell by the
// dataflow kernels (kColourFlow / kColourFlowDense).  What reads only static data or this
// cell's own particles (which no other cell moves) comes first: the cell's list, the
// stencil's layout and the first move's proposal; then `wait()` (the dataflow kernels wait
// there for the earlier-phase neighbours; false: give up), then everything that reads the
// neighbours' particles.
template <bool WL, class Wait>
__device__ __forceinline__ void moveCell(const SweepArgs& a, int cx, int cy, int cz, Wait wait) {
    extern __shared__ float4 dynSmem[];
    __shared__ MoveShared sh;
    float4* candPos = dynSmem;
    int* candIdx = reinterpret_cast<int*>(candPos + kCandCap);
    // FP32 axes of the candidates (stage B), with a surrogate their patch directions as well
    float4* candDir = reinterpret_cast<float4*>(candIdx + kCandCap);
    float4* candPat = a.mlp ? candDir + kCandCap : nullptr;
    const Grid& g = a.g;
    int cell = (cz * g.nc[1] + cy) * g.nc[0] + cx;
    int cnt = a.cellCount[cell];
    if (cnt == 0) return;
    const int tid = threadIdx.x, warp = tid >> 5;
    const double3 box = mk(a.s.box[0], a.s.box[1], a.s.box[2]);
    // the cell's particles: staged in shared memory, or read from the cell list itself when
    // the cell holds more than kCellCap (the list does not change during the sweep)
    const int* list = cnt <= kCellCap ? sh.list : a.cellIdx + a.cellStart[cell];
    if (cnt <= kCellCap)
        for (int k = tid; k < cnt; k += kMoveThreads) sh.list[k] = a.cellIdx[a.cellStart[cell] + k];
    if (tid < 4) sh.propFor[tid] = -1;
    stageStencil(a, cx, cy, cz, sh.st, sh.scan);
    if (warp == 0) buildProposal(a, list, sh.st.nbCell, sh.st.nNb, sh.prop[0], cell, cnt, 0, cx, cy, cz, box);
    else if (tid == 64) acceptThresholds(a, sh.prop[0], cell, 0);
    __syncthreads();
    if (tid == 0) sh.propFor[0] = 0;
    if (!wait()) return;
    if (sh.st.nCand <= kCandCap) loadCandidates(a, sh.st, 0, sh.st.nCand, candIdx, candPos, candDir, candPat);
    const int nCand = sh.st.nCand;
    const bool resident = nCand <= kCandCap;

    DevCtx c;
    c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = a.s.n; c.sqmaxcut = a.t.sqmaxcut;
    const float thr32 = candThreshold(c.sqmaxcut, box);
    double dECell = 0.0;
    unsigned long long nAccT = 0, nRejT = 0, nAccR = 0, nRejR = 0, nTested = 0, nCellRej = 0, nScr = 0;
    unsigned long long nS1Rej = 0, nS2Tried = 0, nS2Rej = 0;
    double daErr2 = 0.0, daErrSum = 0.0;

    // Moves run in passes of one move, or -- with paired passes on and no surrogate stage --
    // of two: move m + 1 is evaluated together with move m, both against the state before
    // move m; queue entries carry the move in bit 1 and the configuration (0 old, 1 new) in
    // bit 0, so the two moves' pairs share the lanes of one stage C.  Move m is decided
    // first; move m + 1's energies stand when move m was rejected or when the two targets
    // are out of each other's range, and its decision is then the one a pass of its own
    // would take (same proposal, same thresholds, same pair energies); otherwise the next
    // pass evaluates it again.  Proposals live in a ring of four slots; warps 2 and 3 build
    // the next pass's during stage C.
    const float bxF = (float)box.x, byF = (float)box.y, bzF = (float)box.z;
    unsigned evalMine = 0;          // pairs this thread evaluated for moves that were decided
    for (int m = 0; m < cnt; ++m) {
        // paired passes start with the second pass (the first builds their proposals)
        const bool pair = !WL && a.pairMoves && !a.mlp && m > 0 && m + 1 < cnt;
        {
            const bool need0 = sh.propFor[m & 3] != m;
            const bool need1 = pair && sh.propFor[(m + 1) & 3] != m + 1;
            if (need0) {
                if (warp == 0) buildProposal(a, list, sh.st.nbCell, sh.st.nNb, sh.prop[m & 3], cell, cnt, m, cx, cy, cz, box);
                else if (tid == 64) acceptThresholds(a, sh.prop[m & 3], cell, m);
            }
            if (need1) {
                if (warp == 1) buildProposal(a, list, sh.st.nbCell, sh.st.nNb, sh.prop[(m + 1) & 3], cell, cnt, m + 1, cx, cy, cz, box);
                else if (tid == 96) acceptThresholds(a, sh.prop[(m + 1) & 3], cell, m + 1);
            }
            __syncthreads();
            if (tid == 0) {
                if (need0) sh.propFor[m & 3] = m;
                if (need1) sh.propFor[(m + 1) & 3] = m + 1;
            }
            __syncthreads();
        }
        const Proposal& P0 = sh.prop[m & 3];
        const Proposal& P1 = sh.prop[(m + 1) & 3];
        if (P0.skip) {
            if (tid == 0) {
                if (P0.displace) { ++nRejT; ++nCellRej; } else ++nRejR;
                countMove(a, P0.type, P0.displace, false);
                if (WL) wlVisit(*a.wl);         // a rejected move visits the current bin
            }
            continue;
        }
        const bool eval1 = pair && !P1.skip;
        const int t = P0.target;
        const bool displace = P0.displace;
        const float3 oldF = P0.oldF, newF = P0.newF;
        const float3 oldF1 = eval1 ? P1.oldF : oldF, newF1 = eval1 ? P1.newF : newF;
        const bool displace1 = eval1 && P1.displace;
        const int t1 = eval1 ? P1.target : -1;

        // delayed acceptance, stage 1: the surrogate's energy change decides first
        float dEs = 0.0f;
        int qaFused = -1;               // >= 0: stage A was fused into the surrogate screen
        if (a.mlp) {
            int partners[4] = {-1, -1, -1, -1};
            for (int q = 0; q < P0.nPartners; ++q) partners[q] = P0.partners[q];
            MovedF mv;
            const PatchSet& ops = a.s.patch[t];
            mv.aOld = f3(P0.odir[0], P0.odir[1], P0.odir[2]);
            mv.pOld = f3(ops.pd[0][0], ops.pd[0][1], ops.pd[0][2]);
            mv.aNew = displace ? mv.aOld : f3(P0.ndir[0], P0.ndir[1], P0.ndir[2]);
            mv.pNew = displace ? mv.pOld : f3(P0.npatch.pd[0][0], P0.npatch.pd[0][1], P0.npatch.pd[0][2]);
            mv.type = P0.type;
            mv.tc = typeCode(mv.type, c.ntypes);
            if (resident) {
                // one pass over the candidates: stage A's screen and the surrogate's
                int* queueS = &sh.queueB[0][0];
                int qa = 0, qs = 0;
                for (int r0 = 0; r0 < nCand; r0 += kMoveThreads) {
                    const int k = r0 + tid;
                    int flags = 0, sflags = 0;
                    if (k < nCand) {
                        int j = candIdx[k];
                        bool partner = (j == partners[0] || j == partners[1] || j == partners[2] || j == partners[3]);
                        if (j != t && !partner) {
                            float4 cp = candPos[k];
                            bool p0 = dist2f(cp, oldF, box) <= thr32;
                            bool p1 = displace ? dist2f(cp, newF, box) <= thr32 : p0;
                            flags = (p0 ? 1 : 0) | (p1 ? 2 : 0);
                            sflags = surrogateScreen(a, mv, cp, candDir[k], displace, oldF, newF, bxF, byF, bzF);
                        }
                    }
                    int total;
                    int off = blockExclusiveScan(__popc(flags) | (__popc(sflags) << 16), total, sh.scan);
                    int oa = off & 0xFFFF, os = off >> 16;
                    if (flags & 1) sh.queueA[qa + oa++] = k << 2;
                    if (flags & 2) sh.queueA[qa + oa] = (k << 2) | 1;
                    if (sflags & 1) queueS[qs + os++] = k << 1;
                    if (sflags & 2) queueS[qs + os] = (k << 1) | 1;
                    qa += total & 0xFFFF;
                    qs += total >> 16;
                }
                __syncthreads();
                dEs = surrogateTotal(sh, surrogateTiles(a, sh, mv, queueS, qs, candPos, candDir, candPat, oldF, newF));
                qaFused = qa;
            } else {
                dEs = surrogateDeltaWindows(a, sh, mv, candIdx, candPos, candDir, candPat, nCand, t, displace, partners,
                                            oldF, newF);
            }
            bool pass = (dEs <= 0.0f) || ((double)dEs < P0.thrStage1);
            if (!pass) {
                if (tid == 0) { ++nS1Rej; if (displace) ++nRejT; else ++nRejR; countMove(a, P0.type, displace, false); }
                __syncthreads();
                continue;
            }
        }

        // energies of move m (0 old, 1 new) and move m + 1 (2 old, 3 new)
        double e0 = 0.0, e1 = 0.0, e2 = 0.0, e3 = 0.0;
        const Con con0 = makeCon(c, t, a.s.mol[t]);
        const Con con1 = eval1 ? makeCon(c, t1, a.s.mol[t1]) : con0;
        auto addE = [&](int b, double en) {
            if (b == 0) e0 += en; else if (b == 1) e1 += en; else if (b == 2) e2 += en; else e3 += en;
        };
        unsigned kept0 = 0, kept1 = 0;
        // bonded partners: both configurations, whatever the distance (warp 0: move m, warp 1: m + 1)
        {
            const int lane = tid & 31;
            const Proposal* Pp = warp == 0 ? &P0 : (warp == 1 && eval1 ? &P1 : nullptr);
            if (Pp && lane < Pp->nPartners) {
                PView b = viewAt(a.s, Pp->partners[lane]);
                const Con& cn = warp == 0 ? con0 : con1;
                unsigned bb; double dd;
                addE(warp * 2, pairEnergy(c, moveView(a.s, *Pp, false), b, cn, box, &bb, &dd));
                addE(warp * 2 + 1, pairEnergy(c, moveView(a.s, *Pp, true), b, cn, box, &bb, &dd));
            }
        }
        int qb0 = 0, qb1 = 0, qb2 = 0;
        // one queue entry through the full pair energy
        auto evalEntry = [&](int q) {
            const Proposal& Pq = (q & 2) ? P1 : P0;
            PView b = viewAt(a.s, candIdx[q >> 2]);
            unsigned bb; double dd;
            addE(q & 3, pairEnergy(c, moveView(a.s, Pq, q & 1), b, (q & 2) ? con1 : con0, box, &bb, &dd));
        };
        // classes 1 and 2 over nw warps starting at warp w0; class 2 starts on a warp boundary
        auto evalGeneric = [&](int w0, int nw) {
            if (warp < w0 || warp >= w0 + nw) return;
            const int pad1 = (qb1 + 31) & ~31;
            for (int g = (warp - w0) * 32 + (tid & 31); g < pad1 + qb2; g += nw * 32) {
                if (g < pad1) { if (g < qb1) evalEntry(sh.queueB[1][g]); }
                else evalEntry(sh.queueB[2][g - pad1]);
            }
        };
        auto evalClass = [&](int cls, int w0, int nw) {     // one class over nw warps from w0
            if (warp < w0 || warp >= w0 + nw) return;
            const int n = cls == 1 ? qb1 : qb2;
            for (int g = (warp - w0) * 32 + (tid & 31); g < n; g += nw * 32) evalEntry(sh.queueB[cls][g]);
        };
        // the next pass's proposals, built while stage C runs: move m + 2 (and m + 3) after a
        // pair, m + 1 otherwise.  They stay valid unless a move of this pass is accepted on the
        // same particle.
        const int specA = pair ? m + 2 : m + 1, specB = pair ? m + 3 : (a.pairMoves && !a.mlp && m == 0 ? m + 2 : cnt);
        auto speculate = [&](int mv) {
            if (sh.propFor[mv & 3] == mv) return;      // still valid from an earlier pass
            Proposal& N = sh.prop[mv & 3];
            buildProposal(a, list, sh.st.nbCell, sh.st.nNb, N, cell, cnt, mv, cx, cy, cz, box);
            if ((tid & 31) == 0) {
                acceptThresholds(a, N, cell, mv);
                sh.propFor[mv & 3] = mv;
            }
        };
        auto flushC = [&](bool last) {     // stage C: exact FP64 pair energies
            __syncthreads();               // queue entries of every thread are visible
            const int lane = tid & 31;
            const bool spec = last && specA < cnt, spec2 = last && specB < cnt;
            if (qb0 > 0) {
                if (warp < 3) {
                    // class 0: warps 0, 1, 2 run the pairs' independent FP64 chains side by side
                    auto getPair = [&](int q, PView& self, PView& other) {
                        self = moveView(a.s, (q & 2) ? P1 : P0, q & 1);
                        other = viewAt(a.s, candIdx[q >> 2]);
                    };
                    for (int r0 = 0; r0 < qb0; r0 += 32) {
                        double e = patchyRound(sh.split, c, box, sh.queueB[0], qb0, r0, getPair);
                        if (warp == 0 && r0 + lane < qb0) addE(sh.queueB[0][r0 + lane] & 3, e);
                    }
                    // the short class-2 pairs (sphere-sphere and others) on warps 1 and 2
                    evalClass(2, 1, 2);
                    if (warp == 2 && spec2) speculate(specB);
                } else {
                    if (spec) speculate(specA);
                    evalClass(1, 3, 1);
                }
            } else if (spec) {
                if (warp == 3) speculate(specA);
                else evalGeneric(0, 3);
                if (warp == 2 && spec2) speculate(specB);
            } else {
                evalGeneric(0, kWarps);
            }
            __syncthreads();
        };
        // stage B over queueA[0, qa): the exact-zero screen in FP32 on the FP32 separation (its
        // margin covers the rounding of the FP32 box fractions).  Pairs it keeps get the full
        // FP64 pair energy, whose own prefilter (r^2 > sqmaxcut) is bit-exact; pairs it drops
        // have energy 0 exactly, so the FP64 prefilter need not run here.
        const float3 dOld0 = f3(P0.odir[0], P0.odir[1], P0.odir[2]), dNew0 = f3(P0.ndir[0], P0.ndir[1], P0.ndir[2]);
        const float3 dOld1 = f3(P1.odir[0], P1.odir[1], P1.odir[2]), dNew1 = f3(P1.ndir[0], P1.ndir[1], P1.ndir[2]);
        auto stageB = [&](int qa) {
            for (int e0_ = 0; e0_ < qa; e0_ += kMoveThreads) {
                int e = e0_ + tid;
                int keep = 0, q = 0, cls = 0;
                if (e < qa) {
                    q = sh.queueA[e];
                    const int k = q >> 2, b = q & 3;
                    float4 cp = candPos[k], cd = candDir[k];
                    const float3 sp = b == 0 ? oldF : (b == 1 ? newF : (b == 2 ? oldF1 : newF1));
                    const float3 sd = b == 0 ? dOld0 : (b == 1 ? dNew0 : (b == 2 ? dOld1 : dNew1));
                    float3 r = pairVecF(sp, cp, bxF, byF, bzF);
                    const PairParam& pp = c.params[((b & 2) ? P1.type : P0.type) * c.ntypes + (int)cp.w];
                    keep = screenedOutF(pp, r, sd, make_float3(cd.x, cd.y, cd.z)) ? 0 : 1;
                    cls = pairClass(pp);
                    if (!keep) ++nScr;
                    else if (b & 2) ++kept1;
                    else ++kept0;
                }
                // one scan, three 10-bit counters: per-class offsets and totals
                int total;
                int off = blockExclusiveScan(keep ? (1 << (10 * cls)) : 0, total, sh.scan);
                if (keep) {
                    int base0 = cls == 0 ? qb0 : (cls == 1 ? qb1 : qb2);
                    sh.queueB[cls][base0 + ((off >> (10 * cls)) & 1023)] = q;
                }
                qb0 += total & 1023;
                qb1 += (total >> 10) & 1023;
                qb2 += (total >> 20) & 1023;
                if (qb0 > kClassCap - kMoveThreads || qb1 > kClassCap - kMoveThreads || qb2 > kClassCap - kMoveThreads) {
                    flushC(false);
                    qb0 = qb1 = qb2 = 0;
                }
            }
        };
        if (qaFused >= 0) {
            stageB(qaFused);
        } else {
            for (int wbase = 0; wbase < nCand; wbase += kCandCap) {
              // candidates in shared memory: all of them, or the window [wbase, wend)
              const int wend = min(wbase + kCandCap, nCand);
              if (!resident) loadCandidates(a, sh.st, wbase, wend - wbase, candIdx, candPos, candDir);
              for (int base = wbase; base < wend; base += kChunk) {
                // stage A: FP32 minimum image against the old and the new position of each move
                int qa = 0;
                const int cend = min(base + kChunk, wend);
                for (int r0 = base; r0 < cend; r0 += kMoveThreads) {
                    int k = r0 + tid - wbase;   // index in the shared-memory window
                    int flags = 0;
                    if (r0 + tid < cend) {
                        int j = candIdx[k];
                        float4 cp = candPos[k];
                        if (j != t && !isPartner(P0, j)) {
                            bool p0 = dist2f(cp, oldF, box) <= thr32;
                            bool p1 = displace ? dist2f(cp, newF, box) <= thr32 : p0;
                            flags = (p0 ? 1 : 0) | (p1 ? 2 : 0);
                        }
                        if (eval1 && j != t1 && !isPartner(P1, j)) {
                            bool p0 = dist2f(cp, oldF1, box) <= thr32;
                            bool p1 = displace1 ? dist2f(cp, newF1, box) <= thr32 : p0;
                            flags |= (p0 ? 4 : 0) | (p1 ? 8 : 0);
                        }
                    }
                    int total;
                    int off = blockExclusiveScan(__popc(flags), total, sh.scan);
#pragma unroll
                    for (int b = 0; b < 4; ++b)
                        if (flags & (1 << b)) sh.queueA[qa + off++] = (k << 2) | b;
                    qa += total;
                }
                __syncthreads();
                stageB(qa);
              }
              if (!resident) {      // queue entries index the window: evaluate them before it changes
                  flushC(false);
                  qb0 = qb1 = qb2 = 0;
              }
            }
        }
        flushC(true);
        blockSum4(e0, e1, e2, e3, sh.red);
        if (tid == 0) {
            // MoveCreator::moveTry (movecreator.h:175-187); with a surrogate stage the exact
            // test is on dE - dEs
            bool accept;
            if (a.mlp) {
                double x = (e1 - e0) - (double)dEs;
                accept = (x <= 0.0) || (x < P0.thrMet);
                ++nS2Tried;
                if (!accept) ++nS2Rej;
                daErr2 += x * x;
                daErrSum += x;
            } else if (WL) {
                // WangLandau::run / runRot (wanglandau.h:124-217): the bins after the move; a
                // bin outside the histogram rejects it, else the weight difference wlener
                // enters moveTry(energy + wlener, enermove) (movecreator.cpp:966-987, 1009-1023)
                WlDev& w = *a.wl;
                long long nw[2], contactsNew;
                double cmNew[3];
                const bool inRange = wlProposal(a, w, P0, box, nw, cmNew, contactsNew);
                double eOld = e0;
                if (inRange) eOld += wlWeight(*w.tab, wlIndex(w, nw)) - wlWeight(*w.tab, wlIndex(w, w.cur));
                accept = inRange && ((e1 <= eOld) || ((e1 - eOld) < P0.thrMet));
                if (accept) {
                    w.cur[0] = nw[0]; w.cur[1] = nw[1];
                    for (int d = 0; d < 3; ++d) w.syscm[d] = cmNew[d];
                    w.contacts = contactsNew;
                }
                wlVisit(w);
            } else {
                accept = (e1 <= e0) || ((e1 - e0) < P0.thrMet);
            }
            nTested += (unsigned long long)nCand * (displace ? 2 : 1);
            evalMine += 2 * P0.nPartners;
            // the accepted state, in global memory and in the cell's staged candidates
            auto commit = [&](const Proposal& P, double dE) {
                const int tt = P.target;
                a.s.pos[tt] = make_double4_32a(P.npos[0], P.npos[1], P.npos[2], (double)P.type);
                if (!P.displace) {
                    a.s.dir[tt] = make_double4_32a(P.ndir[0], P.ndir[1], P.ndir[2], P.dirW);
                    a.s.patch[tt] = P.npatch;
                    float4 nd = make_float4((float)P.ndir[0], (float)P.ndir[1], (float)P.ndir[2], 0.0f);
                    a.cellDirF[a.cellStart[cell] + P.slotR] = nd;
                    if (resident) candDir[sh.st.ownOff + P.slotR] = nd;
                    if (a.mlp) {
                        float4 npd = make_float4((float)P.npatch.pd[0][0], (float)P.npatch.pd[0][1],
                                                 (float)P.npatch.pd[0][2], 0.0f);
                        a.cellPatF[a.cellStart[cell] + P.slotR] = npd;
                        if (resident) candPat[sh.st.ownOff + P.slotR] = npd;
                    }
                    ++nAccR;
                    countMove(a, P.type, false, true);
                } else {
                    countMove(a, P.type, true, true);
                    float4 nf = make_float4(P.newF.x, P.newF.y, P.newF.z, (float)P.type);
                    if (resident) candPos[sh.st.ownOff + P.slotR] = nf;
                    a.cellPosF[a.cellStart[cell] + P.slotR] = nf;
                    ++nAccT;
                }
                dECell += dE;
            };
            // proposals built ahead from a particle this pass moved are stale
            auto invalidate = [&](int after, int tt) {
                for (int q = 0; q < 4; ++q)
                    if (sh.propFor[q] > after && sh.prop[q].target == tt) sh.propFor[q] = -1;
            };
            if (accept) {
                commit(P0, e1 - e0);
                invalidate(m, t);
            } else {
                if (displace) ++nRejT; else ++nRejR;
                countMove(a, P0.type, displace, false);
            }
            int done = 1;
            if (pair) {
                // move m + 1 stands if move m changed nothing it saw
                bool valid = !accept;
                if (!valid && P1.target != t && !isPartner(P1, t)) {
                    float4 o = make_float4(P0.oldF.x, P0.oldF.y, P0.oldF.z, 0.0f);
                    float4 n = make_float4(P0.newF.x, P0.newF.y, P0.newF.z, 0.0f);
                    valid = dist2f(o, P1.oldF, box) > thr32 && dist2f(o, P1.newF, box) > thr32 &&
                            dist2f(n, P1.oldF, box) > thr32 && dist2f(n, P1.newF, box) > thr32;
                }
                if (valid) {
                    done = 2;
                    if (P1.skip) {
                        if (P1.displace) { ++nRejT; ++nCellRej; } else ++nRejR;
                        countMove(a, P1.type, P1.displace, false);
                    } else {
                        nTested += (unsigned long long)nCand * (P1.displace ? 2 : 1);
                        evalMine += 2 * P1.nPartners;
                        if ((e3 <= e2) || ((e3 - e2) < P1.thrMet)) {
                            commit(P1, e3 - e2);
                            invalidate(m + 1, P1.target);
                        } else {
                            if (P1.displace) ++nRejT; else ++nRejR;
                            countMove(a, P1.type, P1.displace, false);
                        }
                    }
                }
            }
            sh.passDone = done;
        }
        __syncthreads();
        const int done = sh.passDone;
        evalMine += kept0 + (done == 2 ? kept1 : 0);
        m += done - 1;
    }
    if (tid == 0) {
        a.cellDE[cell] = dECell;
        atomicAdd(&a.counters[C_ACC_T], nAccT);
        atomicAdd(&a.counters[C_REJ_T], nRejT);
        atomicAdd(&a.counters[C_ACC_R], nAccR);
        atomicAdd(&a.counters[C_REJ_R], nRejR);
        atomicAdd(&a.counters[C_CELL_REJ], nCellRej);
        atomicAdd(&a.counters[C_MOVES], (unsigned long long)cnt);
        atomicAdd(&a.counters[C_TESTED], nTested);
        if (a.mlp) {
            atomicAdd(&a.counters[C_S1_REJ], nS1Rej);
            atomicAdd(&a.counters[C_S2_TRIED], nS2Tried);
            atomicAdd(&a.counters[C_S2_REJ], nS2Rej);
            atomicAdd(&a.ctl->daErr2, daErr2);
            atomicAdd(&a.ctl->daErrSum, daErrSum);
        }
    }
    if (nScr) atomicAdd(&a.counters[C_SCREENED], nScr);
    evalMine = __reduce_add_sync(0xffffffffu, evalMine);
    if ((tid & 31) == 0 && evalMine) atomicAdd(&a.counters[C_EVAL], (unsigned long long)evalMine);
}

// One colour phase: CTA blockIdx.x takes active cell blockIdx.x of the phase's colour.
__device__ __forceinline__ void colourBody(const SweepArgs* __restrict__ A, int phase) {
    const SweepArgs& a = A[blockIdx.y];
    const Grid& g = a.g;
    if ((int)blockIdx.x >= g.nactive || phase >= g.ncolours) return;
    int cx, cy, cz;
    decodeActive(g, a.ctl->perm[phase], blockIdx.x, cx, cy, cz);
    if (a.wl && isWlCell(*a.wl, g, (cz * g.nc[1] + cy) * g.nc[0] + cx)) return;     // moved by kWlCells
    moveCell<false>(a, cx, cy, cz, NoWait());
}

// One CTA per active cell of a colour.  Two register budgets of the same code: kColour
// (up to 255 registers, two CTAs per SM: the shortest move latency, for systems whose
// colours hold few cells) and kColourDense (at most 170 registers, three CTAs per SM:
// more moves in flight per SM, for large systems); the bench's tuner picks one.
__global__ void __launch_bounds__(kMoveThreads, 1) kColour(const SweepArgs* __restrict__ A, int phase) {
    colourBody(A, phase);
}
__global__ void __launch_bounds__(kMoveThreads, 3) kColourDense(const SweepArgs* __restrict__ A, int phase) {
    colourBody(A, phase);
}

// ---- verification of the candidate screens ---------------------------------------------
// For targets i (a list, or every particle) and every other particle j: stage A (the FP32
// candidate screen: wrapped FP32 box fractions, distance^2 against candThreshold) and stage
// B (the FP32 exact-zero screen, screenedOutF on the FP32 separation and axes), computed by
// the same device functions from the same FP32 values as the move kernels (frac32 of the
// FP64 box fractions, as kSortCells and buildProposal make them; FP32 axes as cellDirF).
// Pairs that pass stage A are appended (in no particular order) with their stage-B verdict.
__global__ void kScreenSurvivors(DevState s, DevTables t, const int* targets, int ntargets, long long cap, int* outI,
                                 int* outJ, unsigned char* outB, unsigned long long* count) {
    const double3 box = make_double3(s.box[0], s.box[1], s.box[2]);
    const float thr32 = candThreshold(t.sqmaxcut, box);
    const float bxF = (float)box.x, byF = (float)box.y, bzF = (float)box.z;
    const long long total = (long long)ntargets * s.n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        const int ti = (int)(e / s.n), j = (int)(e - (long long)ti * s.n);
        const int i = targets ? targets[ti] : ti;
        if (i == j) continue;
        const double4_32a pi = s.pos[i], pj = s.pos[j];
        const float3 fi = make_float3(frac32(pi.x), frac32(pi.y), frac32(pi.z));
        const float4 cj = make_float4(frac32(pj.x), frac32(pj.y), frac32(pj.z), (float)pj.w);
        if (!(dist2f(cj, fi, box) <= thr32)) continue;
        const double4_32a di = s.dir[i], dj = s.dir[j];
        const float3 r = pairVecF(fi, cj, bxF, byF, bzF);
        const PairParam& pp = t.params[(int)pi.w * t.ntypes + (int)pj.w];
        const bool keep = !screenedOutF(pp, r, make_float3((float)di.x, (float)di.y, (float)di.z),
                                        make_float3((float)dj.x, (float)dj.y, (float)dj.z));
        const unsigned long long k = atomicAdd(count, 1ull);
        if ((long long)k < cap) { outI[k] = i; outJ[k] = j; outB[k] = keep ? 1 : 0; }
    }
}

// ---- dataflow sweep ---------------------------------------------------------------------
// All colour phases of a sweep in one launch.  CTAs take cells in phase order from a ticket
// counter; a cell first waits until every cell of an earlier phase within its stencil (+-s
// cells per axis: the cells whose particles its moves read, and whose moves read its
// particles) has finished, then moves exactly as in its colour phase.  Cells of one phase
// never touch each other and every pair of cells that does is ordered by phase as the phase
// kernels order it, so each cell sees the states it sees there: the trajectory is the
// phase kernels' (same states, same random numbers), without a grid-wide barrier between
// phases.  Forward progress: a CTA waits only on cells with smaller tickets, taken earlier
// by CTAs that are running, and the smallest unfinished ticket waits on nothing.  Every
// wait is bounded: after a.flowSpin polls (default kFlowSpin) the CTA sets E_FLOW_WAIT and
// every CTA returns; a cell gives up before any of its moves, so every cell of the sweep is
// either moved completely or not at all.
constexpr int kFlowSpin = 1 << 19;      // polls of one wait (~0.2 s; a legitimate wait is < 20 ms)

__device__ __forceinline__ unsigned loadAcquireGpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void storeReleaseGpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <class Wait>
__device__ __forceinline__ void chainCell(const SweepArgs& a, int cx, int cy, int cz, Wait wait);

template <bool CHAIN>
__device__ __forceinline__ void flowBody(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    const Grid& g = a.g;
    if (CHAIN && a.nChains == 0) return;
    const int* counts = CHAIN ? a.chainCellCount : a.cellCount;
    __shared__ int sTicket, sFail;
    __shared__ int posOf[kMaxColours];       // phase of each colour in this sweep
    const int tid = threadIdx.x;
    const unsigned stamp = a.ctl->epoch;
    for (int k = tid; k < g.ncolours; k += kMoveThreads) posOf[a.ctl->perm[k]] = k;
    const int total = g.ncolours * g.nactive;
    const int nx = axisCount(g.nc[0], g.s[0]), ny = axisCount(g.nc[1], g.s[1]), nz = axisCount(g.nc[2], g.s[2]);
    const int nn = nx * ny * nz;
    for (;;) {
        __syncthreads();            // the previous cell's shared state is free; posOf is visible
        if (tid == 0) {
            sTicket = atomicAdd(&a.ctl->ticket, 1);
            sFail = 0;
        }
        __syncthreads();
        const int tk = sTicket;
        if (tk >= total) break;
        const int phase = tk / g.nactive;
        int cx, cy, cz;
        decodeActive(g, a.ctl->perm[phase], tk - phase * g.nactive, cx, cy, cz);
        const int cell = (cz * g.nc[1] + cy) * g.nc[0] + cx;
        // no moves (or, with a Wang-Landau bias, the cells kWlCells moves after the sweep's
        // other cells): nothing to wait for, nothing to publish first
        if (counts[cell] == 0 || (!CHAIN && a.wl && isWlCell(*a.wl, g, cell))) {
            if (tid == 0) storeReleaseGpu(&a.cellDone[cell], stamp);
            continue;
        }
        // the earlier-phase cells of the stencil have finished (false: a wait gave up)
        auto waitNeighbours = [&]() -> bool {
            for (int q = tid; q < nn && !*(volatile int*)&sFail; q += kMoveThreads) {
                int qx = q % nx, qy = (q / nx) % ny, qz = q / (nx * ny);
                int x = axisCell(cx, qx, g.nc[0], g.s[0]);
                int y = axisCell(cy, qy, g.nc[1], g.s[1]);
                int z = axisCell(cz, qz, g.nc[2], g.s[2]);
                int colour = (x % g.p[0]) + g.p[0] * ((y % g.p[1]) + g.p[1] * (z % g.p[2]));
                if (posOf[colour] >= phase) continue;
                const unsigned* f = &a.cellDone[(z * g.nc[1] + y) * g.nc[0] + x];
                for (int spin = 0; loadAcquireGpu(f) != stamp; ++spin) {
                    if (spin >= a.flowSpin || ((spin & 255) == 255 && (*(volatile int*)a.err & E_FLOW_WAIT))) {
                        sFail = 1;
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __syncthreads();
            __threadfence();        // every thread reads the neighbours' states after the waits
            return !sFail;
        };
        if (CHAIN) chainCell(a, cx, cy, cz, waitNeighbours);
        else moveCell<false>(a, cx, cy, cz, waitNeighbours);
        __syncthreads();
        if (sFail) {
            if (tid == 0) atomicOr(a.err, E_FLOW_WAIT);
            break;
        }
        __threadfence();            // each thread's state writes are visible GPU-wide ...
        __syncthreads();
        if (tid == 0) storeReleaseGpu(&a.cellDone[cell], stamp);     // ... before the flag
    }
}

__global__ void __launch_bounds__(kMoveThreads, 1) kColourFlow(const SweepArgs* __restrict__ A) { flowBody<false>(A); }
__global__ void __launch_bounds__(kMoveThreads, 3) kColourFlowDense(const SweepArgs* __restrict__ A) {
    flowBody<false>(A);
}

// ---- one warp per cell ---------------------------------------------------------------------
// The dataflow sweep with a warp, not a CTA, per cell (variant bit 3; plain moves).  A cell of
// a sparse system holds about one particle, so the CTA-wide kernels spend most of a cell's
// time in block barriers and 128-thread scans around a handful of pair energies, with two or
// three cells in flight per SM.  Here each warp takes cells from the sweep's ticket counter on
// its own and runs the same move as moveCell -- the same proposal and threshold streams, the
// same FP32 candidate (stage A) and exact-zero (stage B) screens, the same FP64 pair energy
// -- with warp-synchronous compaction (ballots) and no barrier wider than the warp, so that
// every warp of the SM is an independent cell in flight.  The pair energies of a move are
// summed lane by lane and then over the warp in a fixed order (a different order from
// moveCell's, so the running energies of the two kernels differ in the last bits).  Waiting,
// publishing and the bounded wait are the dataflow sweep's (flowBody).
constexpr int kWarpCand = 256;       // candidates staged per warp at a time (larger stencils: windows)
constexpr int kCellWarps = 4;        // warps per CTA

struct WarpCell {
    float4 candPos[kWarpCand];
    float4 candDir[kWarpCand];
    Proposal prop;
    int candIdx[kWarpCand];
    int queue[2 * kWarpCand];
    int list[kCellCap];
    int nbCell[kNbCap];
    int nbOff[kNbCap + 1];
};
constexpr size_t kDynSmemWarps = sizeof(WarpCell) * kCellWarps;

__device__ __forceinline__ int warpExclusiveScan(int v, int& total) {
    const int lane = threadIdx.x & 31;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

// Sum over the warp in a fixed order (butterfly), the same value in every lane.
__device__ __forceinline__ double warpSumD(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// The moves of one cell by one warp; false when a wait for a neighbour gave up.
__device__ bool warpMoveCell(const SweepArgs& a, WarpCell& W, int cx, int cy, int cz, int cell, int cnt, int phase,
                             const int* posOf, unsigned stamp) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned ltMask = (1u << lane) - 1u;
    const Grid& g = a.g;
    const double3 box = mk(a.s.box[0], a.s.box[1], a.s.box[2]);
    const int start = a.cellStart[cell];
    const int* list = cnt <= kCellCap ? W.list : a.cellIdx + start;     // large cells: the cell list itself
    if (cnt <= kCellCap)
        for (int k = lane; k < cnt; k += 32) W.list[k] = a.cellIdx[start + k];
    // the stencil's cells and their offsets in the candidate list (static during the sweep)
    const int nx = axisCount(g.nc[0], g.s[0]), ny = axisCount(g.nc[1], g.s[1]), nz = axisCount(g.nc[2], g.s[2]);
    const int nn = nx * ny * nz;
    const int ownQ = ((g.nc[2] <= 2 * g.s[2] ? cz : g.s[2]) * ny + (g.nc[1] <= 2 * g.s[1] ? cy : g.s[1])) * nx +
                     (g.nc[0] <= 2 * g.s[0] ? cx : g.s[0]);
    int carry = 0;
    for (int base = 0; base < nn; base += 32) {
        const int q = base + lane;
        int c = 0, cl = 0;
        if (q < nn) {
            const int x = axisCell(cx, q % nx, g.nc[0], g.s[0]);
            const int y = axisCell(cy, (q / nx) % ny, g.nc[1], g.s[1]);
            const int z = axisCell(cz, q / (nx * ny), g.nc[2], g.s[2]);
            cl = (z * g.nc[1] + y) * g.nc[0] + x;
            c = a.cellCount[cl];
        }
        int total;
        const int off = warpExclusiveScan(c, total);
        if (q < nn) { W.nbCell[q] = cl; W.nbOff[q] = carry + off; }
        carry += total;
    }
    if (lane == 0) W.nbOff[nn] = carry;
    __syncwarp();
    const int nCand = carry;
    const int ownOff = W.nbOff[ownQ];
    const bool resident = nCand <= kWarpCand;
    // the first proposal reads only this cell's own particles: built before the wait
    buildProposal(a, list, W.nbCell, nn, W.prop, cell, cnt, 0, cx, cy, cz, box);
    if (lane == 0) acceptThresholds(a, W.prop, cell, 0);
    // the earlier-phase cells of the stencil have finished
    bool fail = false;
    for (int q = lane; q < nn && !fail; q += 32) {
        const int x = axisCell(cx, q % nx, g.nc[0], g.s[0]);
        const int y = axisCell(cy, (q / nx) % ny, g.nc[1], g.s[1]);
        const int z = axisCell(cz, q / (nx * ny), g.nc[2], g.s[2]);
        const int colour = (x % g.p[0]) + g.p[0] * ((y % g.p[1]) + g.p[1] * (z % g.p[2]));
        if (posOf[colour] >= phase) continue;
        const unsigned* f = &a.cellDone[(z * g.nc[1] + y) * g.nc[0] + x];
        for (int spin = 0; loadAcquireGpu(f) != stamp; ++spin) {
            if (spin >= a.flowSpin || ((spin & 255) == 255 && (*(volatile int*)a.err & E_FLOW_WAIT))) {
                fail = true;
                break;
            }
            __nanosleep(64);
        }
    }
    fail = __any_sync(FULL, fail);
    __syncwarp();
    __threadfence();            // every lane reads the neighbours' states after the waits
    if (fail) return false;
    // candidates [first, first + count) of the stencil into the warp's buffers
    auto load = [&](int first, int count) {
        for (int kk = lane; kk < count; kk += 32) {
            const int k = first + kk;
            int lo = 0, hi = nn - 1;          // last q with nbOff[q] <= k
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (W.nbOff[mid] <= k) lo = mid; else hi = mid - 1;
            }
            const int slot = a.cellStart[W.nbCell[lo]] + (k - W.nbOff[lo]);
            W.candIdx[kk] = a.cellIdx[slot];
            W.candPos[kk] = a.cellPosF[slot];
            W.candDir[kk] = a.cellDirF[slot];
        }
        __syncwarp();
    };
    if (resident) load(0, nCand);

    DevCtx c;
    c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = a.s.n; c.sqmaxcut = a.t.sqmaxcut;
    const float thr32 = candThreshold(c.sqmaxcut, box);
    const float bxF = (float)box.x, byF = (float)box.y, bzF = (float)box.z;
    double dECell = 0.0;
    unsigned long long nAccT = 0, nRejT = 0, nAccR = 0, nRejR = 0, nTested = 0, nCellRej = 0;
    unsigned nScr = 0, nEval = 0;
    for (int m = 0; m < cnt; ++m) {
        if (m > 0) {
            buildProposal(a, list, W.nbCell, nn, W.prop, cell, cnt, m, cx, cy, cz, box);
            if (lane == 0) acceptThresholds(a, W.prop, cell, m);
            __syncwarp();
        }
        const Proposal& P = W.prop;
        if (P.skip) {
            if (lane == 0) {
                if (P.displace) { ++nRejT; ++nCellRej; } else ++nRejR;
                countMove(a, P.type, P.displace, false);
            }
            __syncwarp();
            continue;
        }
        const int t = P.target;
        const bool displace = P.displace;
        const float3 oldF = P.oldF, newF = P.newF;
        const float3 dOld = f3(P.odir[0], P.odir[1], P.odir[2]), dNew = f3(P.ndir[0], P.ndir[1], P.ndir[2]);
        const Con con = makeCon(c, t, a.s.mol[t]);
        double e0 = 0.0, e1 = 0.0;
        // bonded partners: both configurations, whatever the distance
        if (lane < P.nPartners) {
            const PView b = viewAt(a.s, P.partners[lane]);
            unsigned bb; double dd;
            e0 += pairEnergy(c, moveView(a.s, P, false), b, con, box, &bb, &dd);
            e1 += pairEnergy(c, moveView(a.s, P, true), b, con, box, &bb, &dd);
        }
        for (int wbase = 0; wbase < nCand; wbase += kWarpCand) {
            const int wend = min(wbase + kWarpCand, nCand);
            if (!resident) load(wbase, wend - wbase);
            // stages A and B: FP32 candidate screen against the old and the new position, then
            // the exact-zero screen on the FP32 separation and axes; survivors compacted
            int qn = 0;
            for (int r0 = wbase; r0 < wend; r0 += 32) {
                const int k = r0 + lane - wbase;
                bool k0 = false, k1 = false;
                if (r0 + lane < wend) {
                    const int j = W.candIdx[k];
                    if (j != t && !isPartner(P, j)) {
                        const float4 cp = W.candPos[k];
                        const bool p0 = dist2f(cp, oldF, box) <= thr32;
                        const bool p1 = displace ? dist2f(cp, newF, box) <= thr32 : p0;
                        if (p0 || p1) {
                            const float4 cd = W.candDir[k];
                            const float3 dj = make_float3(cd.x, cd.y, cd.z);
                            const PairParam& pp = c.params[P.type * c.ntypes + (int)cp.w];
                            if (p0) {
                                k0 = !screenedOutF(pp, pairVecF(oldF, cp, bxF, byF, bzF), dOld, dj);
                                if (!k0) ++nScr;
                            }
                            if (p1) {
                                k1 = !screenedOutF(pp, pairVecF(newF, cp, bxF, byF, bzF), dNew, dj);
                                if (!k1) ++nScr;
                            }
                        }
                    }
                }
                const unsigned b0 = __ballot_sync(FULL, k0), b1 = __ballot_sync(FULL, k1);
                if (k0) W.queue[qn + __popc(b0 & ltMask)] = k << 1;
                if (k1) W.queue[qn + __popc(b0) + __popc(b1 & ltMask)] = (k << 1) | 1;
                qn += __popc(b0) + __popc(b1);
            }
            __syncwarp();
            // stage C: the exact FP64 pair energies, one queue entry per lane
            for (int e = lane; e < qn; e += 32) {
                const int q = W.queue[e];
                const PView b = viewAt(a.s, W.candIdx[q >> 1]);
                unsigned bb; double dd;
                const double en = pairEnergy(c, moveView(a.s, P, q & 1), b, con, box, &bb, &dd);
                if (q & 1) e1 += en; else e0 += en;
                ++nEval;
            }
            __syncwarp();           // the window's buffers are free
        }
        e0 = warpSumD(e0);
        e1 = warpSumD(e1);
        if (lane == 0) {
            // MoveCreator::moveTry (movecreator.h:175-187)
            const bool accept = (e1 <= e0) || ((e1 - e0) < P.thrMet);
            nTested += (unsigned long long)nCand * (displace ? 2 : 1);
            nEval += 2 * P.nPartners;
            if (accept) {
                a.s.pos[t] = make_double4_32a(P.npos[0], P.npos[1], P.npos[2], (double)P.type);
                if (!displace) {
                    a.s.dir[t] = make_double4_32a(P.ndir[0], P.ndir[1], P.ndir[2], P.dirW);
                    a.s.patch[t] = P.npatch;
                    const float4 nd = make_float4((float)P.ndir[0], (float)P.ndir[1], (float)P.ndir[2], 0.0f);
                    a.cellDirF[start + P.slotR] = nd;
                    if (resident) W.candDir[ownOff + P.slotR] = nd;
                    ++nAccR;
                } else {
                    const float4 nf = make_float4(newF.x, newF.y, newF.z, (float)P.type);
                    a.cellPosF[start + P.slotR] = nf;
                    if (resident) W.candPos[ownOff + P.slotR] = nf;
                    ++nAccT;
                }
                dECell += e1 - e0;
            } else {
                if (displace) ++nRejT; else ++nRejR;
            }
            countMove(a, P.type, displace, accept);
        }
        __syncwarp();               // the new state before the next proposal reads it
    }
    if (lane == 0) {
        a.cellDE[cell] = dECell;
        atomicAdd(&a.counters[C_ACC_T], nAccT);
        atomicAdd(&a.counters[C_REJ_T], nRejT);
        atomicAdd(&a.counters[C_ACC_R], nAccR);
        atomicAdd(&a.counters[C_REJ_R], nRejR);
        atomicAdd(&a.counters[C_CELL_REJ], nCellRej);
        atomicAdd(&a.counters[C_MOVES], (unsigned long long)cnt);
        atomicAdd(&a.counters[C_TESTED], nTested);
    }
    nScr = __reduce_add_sync(FULL, nScr);
    nEval = __reduce_add_sync(FULL, nEval);
    if (lane == 0) {
        if (nScr) atomicAdd(&a.counters[C_SCREENED], (unsigned long long)nScr);
        if (nEval) atomicAdd(&a.counters[C_EVAL], (unsigned long long)nEval);
    }
    return true;
}

template <int MINB>
__device__ __forceinline__ void warpFlowBody(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    const Grid& g = a.g;
    extern __shared__ float4 dynSmem[];
    WarpCell& W = reinterpret_cast<WarpCell*>(dynSmem)[threadIdx.x >> 5];
    __shared__ int posOf[kMaxColours];       // phase of each colour in this sweep
    const int lane = threadIdx.x & 31;
    const unsigned stamp = a.ctl->epoch;
    for (int k = threadIdx.x; k < g.ncolours; k += blockDim.x) posOf[a.ctl->perm[k]] = k;
    __syncthreads();
    const int total = g.ncolours * g.nactive;
    for (;;) {
        int tk = 0;
        if (lane == 0) tk = atomicAdd(&a.ctl->ticket, 1);
        tk = __shfl_sync(0xffffffffu, tk, 0);
        if (tk >= total) break;
        const int phase = tk / g.nactive;
        int cx, cy, cz;
        decodeActive(g, a.ctl->perm[phase], tk - phase * g.nactive, cx, cy, cz);
        const int cell = (cz * g.nc[1] + cy) * g.nc[0] + cx;
        const int cnt = a.cellCount[cell];
        if (cnt > 0) {
            if (!warpMoveCell(a, W, cx, cy, cz, cell, cnt, phase, posOf, stamp)) {
                if (lane == 0) atomicOr(a.err, E_FLOW_WAIT);
                break;
            }
            __threadfence();        // each lane's state writes are visible GPU-wide ...
            __syncwarp();
        }
        if (lane == 0) storeReleaseGpu(&a.cellDone[cell], stamp);     // ... before the flag
    }
}

__global__ void __launch_bounds__(kCellWarps * 32, 2) kCellWarpsFlow(const SweepArgs* __restrict__ A) {
    warpFlowBody<2>(A);
}
__global__ void __launch_bounds__(kCellWarps * 32, 3) kCellWarpsFlowDense(const SweepArgs* __restrict__ A) {
    warpFlowBody<3>(A);
}

// ---- Wang-Landau: the order parameters' cells, chain moves, flatness ---------------------
// Sum over particles of volume * position, in a fixed order (block of kMoveThreads): with
// cmK it gives the system centre Conf::syscm as the reference accumulates it (massCenter at
// the start, Conf.cpp:78-95, then + volume * displacement / sysvolume per move).
__device__ void wlCentre(const SweepArgs& a, WlDev& w) {
    __shared__ double red[32][3];
    double s[3] = {0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < a.s.n; i += blockDim.x) {
        const double4_32a p = a.s.pos[i];
        const double v = a.volW[(int)p.w];
        s[0] += v * p.x; s[1] += v * p.y; s[2] += v * p.z;
    }
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[d] += __shfl_down_sync(0xffffffffu, s[d], o);
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; ++d) red[threadIdx.x >> 5][d] = s[d];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int d = 0; d < 3; ++d) {
            double t = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q][d];
            w.syscm[d] = (t - w.cmK[d]) / w.sysvol;
        }
    }
    __syncthreads();
}

// After the colour phases: the sweep's other moves each visited the current bin (they do
// not change the supported order parameters, except order 1 through the system centre,
// which is re-derived here from the positions); then the cells of particles 0 / 1 make their
// moves with the bias, one cell after the other.
__global__ void __launch_bounds__(kMoveThreads, 1) kWlCells(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    if (!a.wl) return;
    WlDev& w = *a.wl;
    const Grid& g = a.g;
    const int slots = wlCellSlots(w, g);
    if (threadIdx.x == 0) {
        long long others = a.s.n;
        for (int k = 0; k < slots; ++k) {
            const int cell = wlCellAt(w, g, k);
            if (cell >= 0) others -= a.cellCount[cell];
        }
        atomicAdd((unsigned long long*)&w.tab->hist[wlIndex(w, w.cur)], (unsigned long long)others);
    }
    if (w.needCM) {
        wlCentre(a, w);
        if (threadIdx.x == 0) {
            long long o[2] = {w.cur[0], w.cur[1]};
            for (int k = 0; k < w.dim; ++k)
                if (w.wlm[k] == 1) o[k] = wlZOrder(w, k, a.s.pos[0].z, w.syscm[2], a.s.box[2]);
            if (wlInRange(w, o)) { w.cur[0] = o[0]; w.cur[1] = o[1]; }
        }
    }
    __syncthreads();
    for (int k = 0; k < slots; ++k) {
        const int cell = wlCellAt(w, g, k);
        if (cell >= 0 && a.cellCount[cell] > 0) {      // an empty cell makes no move
            const int cx = cell % g.nc[0], cy = (cell / g.nc[0]) % g.nc[1], cz = cell / (g.nc[0] * g.nc[1]);
            moveCell<true>(a, cx, cy, cz, NoWait());
        }
        __syncthreads();
    }
}

// After the chain phase: each chain-move attempt visited the current bin.
__global__ void kWlAfterChains(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    if (!a.wl || threadIdx.x != 0 || blockIdx.x != 0) return;
    WlDev& w = *a.wl;
    const unsigned long long seen = a.counters[C_ACC_CH] + a.counters[C_REJ_CH];
    atomicAdd((unsigned long long*)&w.tab->hist[wlIndex(w, w.cur)], seen - w.chainSeen);
    w.chainSeen = seen;
}

// End of a sweep: every kWlUpdateEvery sweeps, WangLandau::update (wanglandau.h:66-120): when
// the smallest bin count exceeds WL_MINHIST and temper * log(max / min) < WL_GERR (max / min
// an integer quotient, as the reference's longs give), alpha is halved, the histogram
// cleared and the weights shifted by the first bin's; below WL_ALPHATOL the run is over.
// A table shared by several walkers is checked by its owner only (the reference's rank 0),
// after every walker's moves of the sweep.
__global__ void kWlEndSweep(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    if (!a.wl || blockIdx.x != 0 || !a.wl->owner) return;
    const WlDev& w = *a.wl;
    WlTable& t = *w.tab;
    if (!(t.alpha > 0.0) || t.converged || a.ctl->sweep % kWlUpdateEvery != 0) return;
    __shared__ long long smin[32], smax[32];
    __shared__ int flat;
    __shared__ double wmin;
    const long long nb = (long long)w.len[0] * w.len[1];
    long long mn = t.hist[0], mx = t.hist[0];
    for (long long i = threadIdx.x; i < nb; i += blockDim.x) {
        mn = min(mn, t.hist[i]);
        mx = max(mx, t.hist[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_down_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = mn; smax[threadIdx.x >> 5] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { mn = min(mn, smin[q]); mx = max(mx, smax[q]); }
        flat = 0;
        if (mn > kWlMinHist && a.temper * log((double)(mx / mn)) < kWlGerr) {
            if (t.alpha < kWlAlphaTol) t.converged = 1;
            else flat = 1;
        }
        wmin = wlWeight(t, 0);
    }
    __syncthreads();
    if (!flat) return;
    for (long long i = threadIdx.x; i < nb; i += blockDim.x) {
        t.base[i] = wlWeight(t, i) - wmin;
        t.hist[i] = 0;
        t.hist0[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        t.alpha /= 2.0;
        t.updates += 1;
    }
}

// Adds the cells' energy changes of this sweep, in a fixed order, and clears them (a cell
// without particles writes nothing during the sweep).
// The sweep's energy change: the per-cell changes summed in a fixed order (each thread a
// strided set of 4-cell groups whose loads are independent, then a shuffle tree per warp,
// the warps in order) and cleared for the next sweep.  One CTA of kEndThreads per system.
constexpr int kEndThreads = 1024;

__global__ void __launch_bounds__(kEndThreads) kEndSweep(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    __shared__ double ws[kEndThreads / 32];
    const int n = a.g.ncells;
    double v = 0.0;
    for (int k0 = (int)threadIdx.x * 4; k0 < n; k0 += kEndThreads * 4) {
        double x[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) x[q] = k0 + q < n ? a.cellDE[k0 + q] : 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v += x[q];
            if (k0 + q < n) a.cellDE[k0 + q] = 0.0;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += ws[q];
        *(a.energyAcc ? a.energyAcc : &a.ctl->energy) += s;
        a.ctl->sweep += 1;
    }
}

// ---- chain moves ---------------------------------------------------------------------------
// MoveCreator::chainMove / chainDisplace / chainRotate / clusterRotate
// (scOOP/mc/movecreator.cpp:305-328, 1075-1256, 1326-1392): a chain (molecule of more than one
// particle) is displaced rigidly by a fixed-length random vector, or rotated about its
// volume-weighted centre by a random quaternion; accepted on mol2others (the chain against
// every particle outside it, empty conlist, totalenergycalculator.h:417-499).
//
// On the GPU the chain moves run in their own checkerboard phase on a coarser grid: a chain
// belongs to the cell holding its centre, cells are at least (maxcut + 2 R)/s wide (R bounds
// |particle - centre| plus the displacement), so chains moved by different cells of one
// colour never come within maxcut of each other; a move whose new centre leaves the cell,
// or whose chain is wider than R, is rejected (both are symmetric in the move).

constexpr int kMaxChain = 20;       // MAXCHL of the reference

__device__ __forceinline__ double3 chainCentre(const SweepArgs& a, int first, int size) {
    double x = 0.0, y = 0.0, z = 0.0, v = 0.0;
    for (int k = 0; k < size; ++k) {      // MoveCreator::clusterCM (movecreator.cpp:1326-1343)
        double4_32a p = a.s.pos[first + k];
        double w = a.volW[(int)p.w];
        x += p.x * w; y += p.y * w; z += p.z * w;
        v += w;
    }
    return mk(x / v, y / v, z / v);
}

// Chains binned by centre into the chain grid (one CTA per system, fixed order in a cell).
__global__ void __launch_bounds__(1024) kChainBin(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    const Grid& g = a.g;
    const Control& ctl = *a.ctl;
    __shared__ int carryS;
    __shared__ int warpS[32];
    for (int c = threadIdx.x; c < g.ncells; c += blockDim.x) { a.chainCellCount[c] = 0; a.cellCursor[c] = 0; }
    __syncthreads();
    for (int ch = threadIdx.x; ch < a.nChains; ch += blockDim.x) {
        int2 fs = a.chains[ch];
        double3 cm = chainCentre(a, fs.x, fs.y);
        int cx = wrapCell(cm.x, ctl.shift[0], g.nc[0]), cy = wrapCell(cm.y, ctl.shift[1], g.nc[1]),
            cz = wrapCell(cm.z, ctl.shift[2], g.nc[2]);
        atomicAdd(&a.chainCellCount[(cz * g.nc[1] + cy) * g.nc[0] + cx], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) carryS = 0;
    __syncthreads();
    for (int base = 0; base < g.ncells; base += blockDim.x) {      // exclusive scan
        int c = base + threadIdx.x;
        int v = c < g.ncells ? a.chainCellCount[c] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) warpS[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int w = warpS[threadIdx.x];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            warpS[threadIdx.x] = w;
        }
        __syncthreads();
        int before = (threadIdx.x >> 5) ? warpS[(threadIdx.x >> 5) - 1] : 0;
        if (c < g.ncells) a.chainCellStart[c] = carryS + before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carryS += before + x;
        __syncthreads();
    }
    for (int ch = threadIdx.x; ch < a.nChains; ch += blockDim.x) {
        int2 fs = a.chains[ch];
        double3 cm = chainCentre(a, fs.x, fs.y);
        int cx = wrapCell(cm.x, ctl.shift[0], g.nc[0]), cy = wrapCell(cm.y, ctl.shift[1], g.nc[1]),
            cz = wrapCell(cm.z, ctl.shift[2], g.nc[2]);
        int cell = (cz * g.nc[1] + cy) * g.nc[0] + cx;
        a.chainCellIdx[a.chainCellStart[cell] + atomicAdd(&a.cellCursor[cell], 1)] = ch;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < g.ncells; c += blockDim.x) {     // ascending chain index
        int* v = a.chainCellIdx + a.chainCellStart[c];
        int n = a.chainCellCount[c];
        for (int i = 1; i < n; ++i) {
            int x = v[i], j = i - 1;
            while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; --j; }
            v[j + 1] = x;
        }
    }
}

struct ChainShared {
    int list[kCellCap];
    int queueA[kQueueCap];
    int queueB[3][kClassCap];
    SplitShared split;
    Stencil st;
    Scan scan;
    double red[kWarps][2];
    int nearIdx[kCandCap];      // candidates within reach of the chain (old or new centre)
    int first, size, displace, skip, constrained;
    double thr;
    double cm[3];
    float3 cmOldF, cmNewF;
    double npos[kMaxChain][3], ndir[kMaxChain][3];
    PatchSet npatch[kMaxChain];
    float3 oldF[kMaxChain], newF[kMaxChain];
};

// Quaternion rotation of a vector (Vector::rotate(Quat), scOOP/structures/Vector.h:162-183).
__device__ __forceinline__ void quatRotate(const double (&q)[4], double* v) {
    double t2 = q[0] * q[1], t3 = q[0] * q[2], t4 = q[0] * q[3], t5 = -q[1] * q[1], t6 = q[1] * q[2],
           t7 = q[1] * q[3], t8 = -q[2] * q[2], t9 = q[2] * q[3], t10 = -q[3] * q[3];
    double x = v[0], y = v[1], z = v[2];
    v[0] = 2.0 * ((t8 + t10) * x + (t6 - t4) * y + (t3 + t7) * z) + x;
    v[1] = 2.0 * ((t4 + t6) * x + (t5 + t10) * y + (t9 - t2) * z) + y;
    v[2] = 2.0 * ((t7 - t3) * x + (t2 + t9) * y + (t5 + t8) * z) + z;
}

// Warp 0: the chain move proposal of move m of this cell.
__device__ void buildChainProposal(const SweepArgs& a, ChainShared& sh, const int* list, int cell, int cnt, int m,
                                   int cx, int cy, int cz, const double3& box) {
    const Control& ctl = *a.ctl;
    const int lane = threadIdx.x & 31;
    const uint32_t sk = (uint32_t)ctl.sweep ^ ((uint32_t)(ctl.sweep >> 32) << 20);
    Stream r(a.seed, (uint32_t)cell, (uint32_t)m, sk);
    int slot = min((int)(r.next() * cnt), cnt - 1);
    int2 fs = a.chains[list[slot]];
    const int first = fs.x, size = min(fs.y, kMaxChain);
    bool displace = r.next() < 0.5;          // chainMove: ran2() < 0.5 displaces
    double3 cm = chainCentre(a, first, size);
    double q[4] = {1.0, 0.0, 0.0, 0.0};
    double dr[3] = {0.0, 0.0, 0.0};
    if (displace) {
        double x, y, z;
        randomUnitSphere(r, x, y, z);
        const int mt = a.s.mol[first].x;
        const double mx = mt < kMaxChainTypes ? a.chainMxType[mt] : a.chainMx;
        dr[0] = x * mx / box.x; dr[1] = y * mx / box.y; dr[2] = z * mx / box.z;
    } else {
        double x, y, z;
        randomUnitSphere(r, x, y, z);
        double vc = cos(a.chainAngle * r.next());
        double vs = (r.next() < 0.5) ? sqrt(1.0 - vc * vc) : -sqrt(1.0 - vc * vc);
        q[0] = vc; q[1] = x * vs; q[2] = y * vs; q[3] = z * vs;
    }
    int wide = 0;
    if (lane < size) {
        const int i = first + lane;
        double4_32a p = a.s.pos[i], d = a.s.dir[i];
        double v[3] = {p.x, p.y, p.z};
        double rx = (p.x - cm.x) * box.x, ry = (p.y - cm.y) * box.y, rz = (p.z - cm.z) * box.z;
        wide = (rx * rx + ry * ry + rz * rz > a.chainR * a.chainR);
        double dd[3] = {d.x, d.y, d.z};
        if (displace) {
            for (int k = 0; k < 3; ++k) v[k] += dr[k];
        } else {
            // clusterRotate: shift to the centre, scale by the box, rotate, scale back, shift back
            for (int k = 0; k < 3; ++k) v[k] -= (&cm.x)[k];
            v[0] *= box.x; v[1] *= box.y; v[2] *= box.z;
            quatRotate(q, v);
            v[0] /= box.x; v[1] /= box.y; v[2] /= box.z;
            for (int k = 0; k < 3; ++k) v[k] += (&cm.x)[k];
            quatRotate(q, dd);
            const PatchSet& ps = a.s.patch[i];
            PatchSet& np = sh.npatch[lane];
            for (int u = 0; u < 2; ++u) { double w[3] = {ps.pd[u][0], ps.pd[u][1], ps.pd[u][2]}; quatRotate(q, w); for (int k = 0; k < 3; ++k) np.pd[u][k] = w[k]; }
            for (int u = 0; u < 2; ++u) { double w[3] = {ps.ch[u][0], ps.ch[u][1], ps.ch[u][2]}; quatRotate(q, w); for (int k = 0; k < 3; ++k) np.ch[u][k] = w[k]; }
            for (int u = 0; u < 4; ++u) { double w[3] = {ps.ps[u][0], ps.ps[u][1], ps.ps[u][2]}; quatRotate(q, w); for (int k = 0; k < 3; ++k) np.ps[u][k] = w[k]; }
        }
        for (int k = 0; k < 3; ++k) { sh.npos[lane][k] = v[k]; sh.ndir[lane][k] = dd[k]; }
        sh.oldF[lane] = make_float3(frac32(p.x), frac32(p.y), frac32(p.z));
        sh.newF[lane] = make_float3(frac32(v[0]), frac32(v[1]), frac32(v[2]));
    }
    wide = __any_sync(0xffffffffu, wide);
    __syncwarp();
    if (lane == 0) {
        // the new centre (from the new positions, as for the reverse move) must stay in the cell
        double x = 0.0, y = 0.0, z = 0.0, vv = 0.0;
        for (int k = 0; k < size; ++k) {
            double w = a.volW[(int)a.s.pos[first + k].w];
            x += sh.npos[k][0] * w; y += sh.npos[k][1] * w; z += sh.npos[k][2] * w;
            vv += w;
        }
        x /= vv; y /= vv; z /= vv;
        bool inside = wrapCell(x, ctl.shift[0], a.g.nc[0]) == cx && wrapCell(y, ctl.shift[1], a.g.nc[1]) == cy &&
                      wrapCell(z, ctl.shift[2], a.g.nc[2]) == cz;
        sh.first = first;
        sh.size = size;
        sh.displace = displace;
        sh.cmOldF = make_float3(frac32(cm.x), frac32(cm.y), frac32(cm.z));
        sh.cmNewF = make_float3(frac32(x), frac32(y), frac32(z));
        sh.skip = (!inside || wide) ? 1 : 0;
        sh.constrained = wide ? 1 : 0;
        Stream ru(a.seed ^ 0xD1B54A32D192ED03ull, (uint32_t)cell, (uint32_t)m, sk);
        sh.thr = -a.temper * log(ru.next());
    }
}

// One CTA per active cell of the chain grid: that cell's chain moves in sequence (stages
// A, B, C as in kColour over (chain particle, candidate) pairs, old and new configuration).
// The chain moves of chain cell (cx, cy, cz), by the whole CTA (kChainColour: one colour
// phase; kChainFlow: the dataflow sweep of the chain grid, which waits in `wait()` after the
// static layout is staged; false: give up).
template <class Wait>
__device__ __forceinline__ void chainCell(const SweepArgs& a, int cx, int cy, int cz, Wait wait) {
    extern __shared__ float4 dynSmem[];
    __shared__ ChainShared sh;
    float4* candPos = dynSmem;
    int* candIdx = reinterpret_cast<int*>(candPos + kCandCap);
    const Control& ctl = *a.ctl;
    const Grid& g = a.g;
    const int cell = (cz * g.nc[1] + cy) * g.nc[0] + cx;
    const int cnt = a.chainCellCount[cell];
    if (cnt == 0) return;
    const int tid = threadIdx.x;
    // attempts of this cell this sweep: cnt * chainFrac, the fraction rounded at random
    Stream rm(a.seed ^ 0x9E3779B97F4A7C15ull, (uint32_t)cell, 0xC4A1u,
              (uint32_t)ctl.sweep ^ ((uint32_t)(ctl.sweep >> 32) << 20));
    const double want = cnt * a.chainFrac;
    const int moves = (int)want + ((rm.next() < want - floor(want)) ? 1 : 0);
    if (moves == 0) return;
    // the cell's chains: staged in shared memory, or read from the chain list itself when the
    // cell holds more than kCellCap
    const int* list = cnt <= kCellCap ? sh.list : a.chainCellIdx + a.chainCellStart[cell];
    if (cnt <= kCellCap)
        for (int k = tid; k < cnt; k += kMoveThreads) sh.list[k] = a.chainCellIdx[a.chainCellStart[cell] + k];
    stageStencil(a, cx, cy, cz, sh.st, sh.scan);
    if (!wait()) return;
    const int nCand = sh.st.nCand;
    const bool resident = nCand <= kCandCap;
    if (resident) loadCandidates(a, sh.st, 0, nCand, candIdx, candPos);
    const int warp = tid >> 5;
    DevCtx c;
    c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = a.s.n; c.sqmaxcut = a.t.sqmaxcut;
    const Con con = emptyCon(c);
    const double3 box = mk(a.s.box[0], a.s.box[1], a.s.box[2]);
    const float thr32 = candThreshold(c.sqmaxcut, box);
    const float reachNear = sqrtf(thr32) + (float)a.chainR + 1e-3f;
    const float thrNear = reachNear * reachNear * 1.0001f;
    double dECell = 0.0;
    unsigned long long nAcc = 0, nRej = 0, nConstr = 0, nTested = 0, nEval = 0;

    for (int m = 0; m < moves; ++m) {
        if (tid < 32) buildChainProposal(a, sh, list, cell, cnt, m, cx, cy, cz, box);
        __syncthreads();
        if (sh.skip) {
            if (tid == 0) { ++nRej; nConstr += sh.constrained; }
            __syncthreads();
            continue;
        }
        const int first = sh.first, size = sh.size;
        const bool displace = sh.displace;
        auto view = [&](int i, bool isNew) {
            PView v = viewAt(a.s, first + i);
            if (isNew) {
                v.pos = mk(sh.npos[i][0], sh.npos[i][1], sh.npos[i][2]);
                v.dir = mk(sh.ndir[i][0], sh.ndir[i][1], sh.ndir[i][2]);
                if (!displace) v.patch = &sh.npatch[i];
            }
            return v;
        };
        double eOld = 0.0, eNew = 0.0;
        int qb0 = 0, qb1 = 0, qb2 = 0;
        auto getPair = [&](int q, PView& self, PView& other) {
            self = view((q >> 1) % kMaxChain, q & 1);
            other = viewAt(a.s, (q >> 1) / kMaxChain);
        };
        auto evalEntry = [&](int q) {
            PView self, other;
            getPair(q, self, other);
            unsigned bb; double dd;
            double en = pairEnergy(c, self, other, con, box, &bb, &dd);
            if (q & 1) eNew += en; else eOld += en;
        };
        auto evalClass = [&](int cls, int w0, int nw) {     // one class over nw warps from w0
            if (warp < w0 || warp >= w0 + nw) return;
            const int n = cls == 1 ? qb1 : qb2;
            for (int g = (warp - w0) * 32 + (tid & 31); g < n; g += nw * 32) evalEntry(sh.queueB[cls][g]);
        };
        // stage C as in kColour: patchy SC-SC pairs as parallel chains on warps 0-2,
        // SC-sphere pairs on warp 3, the rest on warps 1-2 afterwards
        auto flushC = [&]() {
            __syncthreads();
            if (qb0 > 0) {
                if (warp < 3) {
                    for (int r0 = 0; r0 < qb0; r0 += 32) {
                        double en = patchyRound(sh.split, c, box, sh.queueB[0], qb0, r0, getPair);
                        if (warp == 0 && r0 + (tid & 31) < qb0) {
                            if (sh.queueB[0][r0 + (tid & 31)] & 1) eNew += en; else eOld += en;
                        }
                    }
                    evalClass(2, 1, 2);
                } else {
                    evalClass(1, 3, 1);
                }
            } else {
                evalClass(1, 0, 2);
                evalClass(2, 2, 2);
            }
            __syncthreads();
            nEval += qb0 + qb1 + qb2;
            qb0 = qb1 = qb2 = 0;
        };
        for (int wbase = 0; wbase < nCand; wbase += kCandCap) {
            const int wlen = min(kCandCap, nCand - wbase);
            if (!resident) loadCandidates(a, sh.st, wbase, wlen, candIdx, candPos);
            // stage A0: the candidates within chainR + cut-off of the old or the new centre
            // (every chain particle lies within chainR of its centre), outside the chain
            int nNear = 0;
            for (int r0 = 0; r0 < wlen; r0 += kMoveThreads) {
                int k = r0 + tid, flag = 0;
                if (k < wlen) {
                    int j = candIdx[k];
                    if (j < first || j >= first + size) {
                        float4 cp = candPos[k];
                        flag = (dist2f(cp, sh.cmOldF, box) <= thrNear || dist2f(cp, sh.cmNewF, box) <= thrNear) ? 1 : 0;
                    }
                }
                int tot;
                int off = blockExclusiveScan(flag, tot, sh.scan);
                if (flag) sh.nearIdx[nNear + off] = k;
                nNear += tot;
            }
            __syncthreads();
            const int total = nNear * size;
            for (int base = 0; base < total; base += kChunk) {
                const int end = min(base + kChunk, total);
                int qa = 0;
                for (int r0 = base; r0 < end; r0 += kMoveThreads) {     // stage A
                    int idx = r0 + tid, flags = 0, k = 0, pi = 0;
                    if (idx < end) {
                        int kk = idx / size;
                        pi = idx - kk * size;
                        k = sh.nearIdx[kk];
                        float4 cp = candPos[k];
                        bool p0 = dist2f(cp, sh.oldF[pi], box) <= thr32;
                        bool p1 = dist2f(cp, sh.newF[pi], box) <= thr32;
                        flags = (p0 ? 1 : 0) | (p1 ? 2 : 0);
                    }
                    int tot;
                    int off = blockExclusiveScan(__popc(flags), tot, sh.scan);
                    // entries name the particle, not the window slot: stage C runs once
                    // over all windows
                    int key = flags ? ((candIdx[k] * kMaxChain + pi) << 1) : 0;
                    if (flags & 1) sh.queueA[qa + off++] = key;
                    if (flags & 2) sh.queueA[qa + off] = key | 1;
                    qa += tot;
                }
                __syncthreads();
                for (int e0 = 0; e0 < qa; e0 += kMoveThreads) {             // stage B
                    int e = e0 + tid, keep = 0, q = 0, cls = 0;
                    if (e < qa) {
                        q = sh.queueA[e];
                        int isNew = q & 1, pi = (q >> 1) % kMaxChain, j = (q >> 1) / kMaxChain;
                        PView self = view(pi, isNew);
                        double4_32a pj = a.s.pos[j];
                        double3 r = imageVec(self.pos, mk(pj.x, pj.y, pj.z), box);
                        if (!(dot3(r, r) > c.sqmaxcut)) {
                            double4_32a dj = a.s.dir[j];
                            const PairParam& pp = c.params[self.type * c.ntypes + (int)pj.w];
                            keep = screenedOut(pp, r, self.dir, mk(dj.x, dj.y, dj.z)) ? 0 : 1;
                            cls = pairClass(pp);
                        }
                    }
                    int tot;
                    int off = blockExclusiveScan(keep ? (1 << (10 * cls)) : 0, tot, sh.scan);
                    if (keep) {
                        int base0 = cls == 0 ? qb0 : (cls == 1 ? qb1 : qb2);
                        sh.queueB[cls][base0 + ((off >> (10 * cls)) & 1023)] = q;
                    }
                    qb0 += tot & 1023;
                    qb1 += (tot >> 10) & 1023;
                    qb2 += (tot >> 20) & 1023;
                    if (qb0 > kClassCap - kMoveThreads || qb1 > kClassCap - kMoveThreads || qb2 > kClassCap - kMoveThreads)
                        flushC();
                }
            }
        }
        flushC();
        nTested += (unsigned long long)nCand * size * 2;
        blockSum2(eOld, eNew, sh.red);
        __shared__ int acceptS;
        if (tid == 0) {
            double dE = eNew - eOld;
            bool accept = (dE <= 0.0) || (dE < sh.thr);
            acceptS = accept;
            if (accept) { dECell += dE; ++nAcc; } else ++nRej;
            const int mt = a.s.mol[first].x;
            if (a.typeCtr && mt < kMaxChainTypes)
                atomicAdd(&a.typeCtr[kTypeCtrChain + 4 * mt + (displace ? 0 : 2) + (accept ? 0 : 1)], 1ull);
        }
        __syncthreads();
        if (acceptS && tid < size) {
            const int i = first + tid;
            double4_32a p = a.s.pos[i];
            a.s.pos[i] = make_double4_32a(sh.npos[tid][0], sh.npos[tid][1], sh.npos[tid][2], p.w);
            if (!displace) {
                double4_32a d = a.s.dir[i];
                a.s.dir[i] = make_double4_32a(sh.ndir[tid][0], sh.ndir[tid][1], sh.ndir[tid][2], d.w);
                a.s.patch[i] = sh.npatch[tid];
            }
            // the particle's entry in this grid's cell list (and in shared memory)
            const int pc = a.cellOf[i], slot = a.slotOf[i];
            float4 nf = make_float4(sh.newF[tid].x, sh.newF[tid].y, sh.newF[tid].z, (float)p.w);
            a.cellPosF[slot] = nf;
            if (resident)
                for (int q = 0; q < sh.st.nNb; ++q)
                    if (sh.st.nbCell[q] == pc) candPos[sh.st.nbOff[q] + (slot - a.cellStart[pc])] = nf;
        }
        __syncthreads();
    }
    if (tid == 0) {
        a.cellDE[cell] = dECell;
        atomicAdd(&a.counters[C_ACC_CH], nAcc);
        atomicAdd(&a.counters[C_REJ_CH], nRej);
        if (nConstr) atomicAdd(&a.counters[C_CH_CONSTR], nConstr);
        atomicAdd(&a.counters[C_TESTED], nTested);
        atomicAdd(&a.counters[C_EVAL], nEval);
    }
}

// One colour phase of the chain grid: CTA blockIdx.x takes active chain cell blockIdx.x.
__global__ void __launch_bounds__(kMoveThreads, 1) kChainColour(const SweepArgs* __restrict__ A, int phase) {
    const SweepArgs& a = A[blockIdx.y];
    const Grid& g = a.g;
    if (a.nChains == 0 || (int)blockIdx.x >= g.nactive || phase >= g.ncolours) return;
    int cx, cy, cz;
    decodeActive(g, a.ctl->perm[phase], blockIdx.x, cx, cy, cz);
    chainCell(a, cx, cy, cz, NoWait());
}

// The chain grid's dataflow sweep: chains centred in cells of one colour are more than
// maxcut apart whatever they do (cells >= (maxcut + 2 (R + displacement)) / 2), and a chain
// cell can only interact with chain cells within +-2 cells -- the stencil the flow waits on.
__global__ void __launch_bounds__(kMoveThreads, 1) kChainFlow(const SweepArgs* __restrict__ A) { flowBody<true>(A); }

// Largest |particle - chain centre| (real space) over all chains, as float bits (>= 0).
__global__ void kChainExtent(SweepArgs a, const int2* chains, int nChains, unsigned* out) {
    int ch = blockIdx.x * blockDim.x + threadIdx.x;
    if (ch >= nChains) return;
    int2 fs = chains[ch];
    double3 cm = chainCentre(a, fs.x, fs.y);
    double m = 0.0;
    for (int k = 0; k < fs.y; ++k) {
        double4_32a p = a.s.pos[fs.x + k];
        double x = (p.x - cm.x) * a.s.box[0], y = (p.y - cm.y) * a.s.box[1], z = (p.z - cm.z) * a.s.box[2];
        m = fmax(m, sqrt(x * x + y * y + z * z));
    }
    atomicMax(out, __float_as_uint((float)m));
}

// The cell-energy kernel runs one warp per cell (many cells in flight per SM: a cell holds
// a few particles and a few pairs in range, so the staging latency, not the arithmetic,
// sets its time), with candidate windows of kCellCandCap and queues of kCellQueueCap.
constexpr int kCellThreads = 32;
constexpr int kCellCandCap = 256;
constexpr int kCellQueueCap = 512;
constexpr size_t kDynSmemCell = (size_t)kCellCandCap * (sizeof(float4) + sizeof(int));

struct CellShared {
    int list[kCellCap];
    int queueA[kCellQueueCap];
    int queueB[kCellQueueCap];
    Stencil st;
    Scan scan;
};

// Total energy over the cell list, one CTA per cell: PairE(i, j, conlist(i)) for every
// particle i of the cell and j < i (allToAll's pair orientation,
// totalenergycalculator.h:502-521), with the same A/B/C stages as the move kernel.
__global__ void __launch_bounds__(kCellThreads) kCellEnergy(const SweepArgs* __restrict__ A, int useTrialBox) {
    extern __shared__ float4 dynSmem[];
    float4* candPos = dynSmem;
    int* candIdx = reinterpret_cast<int*>(candPos + kCellCandCap);
    __shared__ CellShared sh;
    const SweepArgs& a = A[blockIdx.y];
    const Control& ctl = *a.ctl;
    const Grid& g = a.g;
    const int cell = blockIdx.x;
    const int tid = threadIdx.x;
    if (cell >= g.ncells) return;
    if (useTrialBox && !ctl.volValid) {
        if (tid == 0) a.partial[cell] = 0.0;
        return;
    }
    int cnt = a.cellCount[cell];
    if (cnt == 0) {
        if (tid == 0) a.partial[cell] = 0.0;
        return;
    }
    int cx = cell % g.nc[0], cy = (cell / g.nc[0]) % g.nc[1], cz = cell / (g.nc[0] * g.nc[1]);
    const int own0 = a.cellStart[cell];
    const int* list = cnt <= kCellCap ? sh.list : a.cellIdx + own0;      // large cells: the cell list itself
    if (cnt <= kCellCap)
        for (int k = tid; k < cnt; k += kCellThreads) sh.list[k] = a.cellIdx[own0 + k];
    stageStencil<kCellThreads>(a, cx, cy, cz, sh.st, sh.scan);
    const int nCand = sh.st.nCand;
    DevCtx c;
    c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = a.s.n; c.sqmaxcut = a.t.sqmaxcut;
    const double* bx = useTrialBox ? ctl.trialBox : a.s.box;
    const double3 box = mk(bx[0], bx[1], bx[2]);
    const float thr32 = candThreshold(c.sqmaxcut, box);
    double sum = 0.0;
    // bonded partners j < i, whatever the distance
    for (int k = tid; k < cnt; k += kCellThreads) {
        int i = list[k];
        Con con = makeCon(c, i, a.s.mol[i]);
        PView vi = viewAt(a.s, i);
        for (int q = 0; q < 4; ++q) {
            int j = con.idx[q];
            if (j >= 0 && j < i) {
                unsigned bb; double dd;
                sum += pairEnergy(c, vi, viewAt(a.s, j), con, box, &bb, &dd);
            }
        }
    }
    int qb = 0, wlen = 0;
    auto flushC = [&](int count) {
        __syncthreads();                   // queue entries of every thread are visible
        for (int e = tid; e < count; e += kCellThreads) {
            int q = sh.queueB[e];
            int i = list[q / wlen], j = candIdx[q % wlen];
            Con con = makeCon(c, i, a.s.mol[i]);
            unsigned bb; double dd;
            sum += pairEnergy(c, viewAt(a.s, i), viewAt(a.s, j), con, box, &bb, &dd);
        }
        __syncthreads();
    };
    for (int wbase = 0; wbase < nCand; wbase += kCellCandCap) {
      // the candidates in windows of kCellCandCap; pair q = (own particle li, window slot k)
      wlen = min(kCellCandCap, nCand - wbase);
      loadCandidates<kCellThreads>(a, sh.st, wbase, wlen, candIdx, candPos);
      const int total = cnt * wlen;
      for (int base = 0; base < total; base += kChunk) {
        int qa = 0;
        int end = min(base + kChunk, total);
        for (int r0 = base; r0 < end; r0 += kCellThreads) {
            int q = r0 + tid;
            int keep = 0;
            if (q < end) {
                int li = q / wlen, k = q % wlen;
                int i = list[li], j = candIdx[k];
                if (j < i) {
                    float4 pi = a.cellPosF[own0 + li];
                    keep = dist2f(candPos[k], make_float3(pi.x, pi.y, pi.z), box) <= thr32;
                }
            }
            int tot;
            int off = blockExclusiveScan<kCellThreads>(keep, tot, sh.scan);
            if (keep) sh.queueA[qa + off] = q;
            qa += tot;
        }
        __syncthreads();
        for (int e0 = 0; e0 < qa; e0 += kCellThreads) {
            int e = e0 + tid;
            int keep = 0, q = 0;
            if (e < qa) {
                q = sh.queueA[e];
                int i = list[q / wlen], j = candIdx[q % wlen];
                int4 mi = a.s.mol[i];
                Con con = makeCon(c, i, mi);
                bool partner = (j == con.idx[0] || j == con.idx[1] || j == con.idx[2] || j == con.idx[3]);
                if (!partner) {
                    double4_32a pi = a.s.pos[i], pj = a.s.pos[j];
                    double3 r = imageVec(mk(pi.x, pi.y, pi.z), mk(pj.x, pj.y, pj.z), box);
                    if (!(dot3(r, r) > c.sqmaxcut)) {
                        double4_32a di = a.s.dir[i], dj = a.s.dir[j];
                        const PairParam& pp = c.params[(int)pi.w * c.ntypes + (int)pj.w];
                        keep = screenedOut(pp, r, mk(di.x, di.y, di.z), mk(dj.x, dj.y, dj.z)) ? 0 : 1;
                    }
                }
            }
            int tot;
            int off = blockExclusiveScan<kCellThreads>(keep, tot, sh.scan);
            if (keep) sh.queueB[qb + off] = q;
            qb += tot;
            if (qb > kCellQueueCap - kCellThreads) { flushC(qb); qb = 0; }
        }
      }
      flushC(qb);           // queue entries index the window
      qb = 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);     // fixed order
    if (tid == 0) a.partial[cell] = sum;
}

// Sum of the per-cell partials p[0, n) by all threads of one block in a fixed order (strided
// per-thread sums, a shuffle tree per warp, the warps in order): every thread gets the same
// value, launch after launch.  A single-thread loop over the 3000+ cells of a small system
// is a dependent FP64 chain of ~0.1 ms.
__device__ double sumPartials(const double* p, int n) {
    __shared__ double ws[32];
    double v = 0.0;
    const int stride = (int)blockDim.x * 8;
    for (int k0 = (int)threadIdx.x * 8; k0 < n; k0 += stride) {     // 8 independent loads a thread
        double x[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) x[q] = k0 + q < n ? p[k0 + q] : 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q) v += x[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += ws[q];
    return s;
}

// MoveCreator::pressureMove, ptype 1 (movecreator.cpp:390-421), decided on the device.
// Wang-Landau order 7 in a trial box (runPress calls contParticlesAll, wanglandau.h:603-615):
// the particles 1..N-1 of the counted type within the contact distance of particle 0,
// counted by the whole block (integer sums: the order of the additions does not matter).
__device__ long long wlContactsBlock(const SweepArgs& a, const WlDev& w, const double* box) {
    __shared__ unsigned long long tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    const double4_32a q0 = a.s.pos[0];
    const double p0[3] = {q0.x, q0.y, q0.z};
    unsigned long long n = 0;
    for (int i = 1 + (int)threadIdx.x; i < a.s.n; i += blockDim.x) {
        const double4_32a q = a.s.pos[i];
        const double pi[3] = {q.x, q.y, q.z};
        if ((int)q.w == w.contactType && wlInContact(pi, p0, box)) ++n;
    }
    if (n) atomicAdd(&tot, n);
    __syncthreads();
    return (long long)tot;
}

__global__ void kVolumeAccept(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    if (blockIdx.x != 0) return;
    Control& c = *a.ctl;
    if (!c.volValid) {
        if (threadIdx.x == 0) {
            atomicAdd(&a.counters[C_VOL_CONSTR], 1ull);
            atomicAdd(&a.counters[C_REJ_V], 1ull);
            if (a.wl) wlVisit(*a.wl);
        }
        return;
    }
    double eNew = sumPartials(a.partial, a.g.ncells);
    if (a.wl && a.wl->needCM) wlCentre(a, *a.wl);
    const long long contactsTrial = a.wl && a.wl->useContacts ? wlContactsBlock(a, *a.wl, c.trialBox) : 0;
    if (threadIdx.x != 0) return;
    double enermove = c.pvTerm;
    enermove += eNew;
    Stream r(a.seed, 0xFFFFFFF1u, (uint32_t)c.sweep, (uint32_t)(c.sweep >> 32));
    double u = r.next();
    double energy = c.energy;
    long long nw[2];
    bool inRange = true;
    if (a.wl) {
        // WangLandau::runPress (wanglandau.h:168-196) with the trial box: order 1 (not for
        // ptype 2, whose z stays), 4, the contacts 7 and the box lengths 8 / 9 change; wlener
        // enters moveTry(energy + wlener, enermove)
        WlDev& w = *a.wl;
        const double* tb = c.trialBox;
        nw[0] = w.cur[0]; nw[1] = w.cur[1];
        for (int k = 0; k < w.dim; ++k) {
            switch (w.wlm[k]) {
            case 1:
                if (a.ptype != 2) nw[k] = wlZOrder(w, k, a.s.pos[0].z, w.syscm[2], tb[2]);
                break;
            case 4: {
                const double4_32a q0 = a.s.pos[0], q1 = a.s.pos[1];
                const double p0[3] = {q0.x, q0.y, q0.z}, p1[3] = {q1.x, q1.y, q1.z};
                nw[k] = wlDistOrder(w, k, p0, p1, tb);
                break;
            }
            case 7: nw[k] = wlContactOrder(w, k, contactsTrial); break;
            case 8: nw[k] = wlBoxOrder(w, k, tb[0]); break;
            case 9: nw[k] = wlBoxOrder(w, k, tb[1]); break;
            default: break;
            }
        }
        inRange = wlInRange(w, nw);
        if (inRange) energy += wlWeight(*w.tab, wlIndex(w, nw)) - wlWeight(*w.tab, wlIndex(w, w.cur));
    }
    bool accept = inRange && ((enermove <= energy) || (exp(-1.0 * (enermove - energy) / a.temper) > u));
    if (accept) {
        for (int d = 0; d < 3; ++d) a.s.box[d] = c.trialBox[d];
        c.energy = eNew;
        atomicAdd(&a.counters[C_ACC_V], 1ull);
        if (a.wl) {
            a.wl->cur[0] = nw[0]; a.wl->cur[1] = nw[1];
            if (a.wl->useContacts) a.wl->contacts = contactsTrial;
        }
    } else {
        atomicAdd(&a.counters[C_REJ_V], 1ull);
    }
    if (a.wl) wlVisit(*a.wl);
}

__global__ void kSetEnergy(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    if (blockIdx.x != 0) return;
    double e = sumPartials(a.partial, a.g.ncells);
    if (threadIdx.x == 0) a.ctl->energy = e;
}

__global__ void kCheckEnergy(const SweepArgs* __restrict__ A) {
    const SweepArgs& a = A[blockIdx.y];
    if (blockIdx.x != 0) return;
    double e = sumPartials(a.partial, a.g.ncells);
    if (threadIdx.x != 0) return;
    Control& c = *a.ctl;
    c.energyCheck = e;
    double d = fabs(c.energy - e);
    if (d > c.maxDrift) c.maxDrift = d;
}


// Replica exchange (MoveCreator::replicaExchangeMove, scOOP/mc/movecreator.cpp:552-795,
// there over MPI): within each ladder the even and the odd neighbour pairs of the
// temperature ladder are tried alternately; a swap of temperatures between the replica
// at rank k (colder) and the one at rank k+1 is accepted with
// min(1, exp((1/T_k - 1/T_k+1)(E_k - E_k+1) + (P_k/T_k - P_k+1/T_k+1)(V_k - V_k+1))),
// the canonical plus isobaric rule of the reference (the pressure term vanishes in NVT).
__device__ double gcExchangeTerm(const SweepArgs& ai, const SweepArgs& aj, double Ti, double Tj);

__global__ void kExchange(SweepArgs* A, SweepArgs* AC, int* ladder, const int* ladderStart, int nLadders,
                          uint64_t seed, unsigned long long* ctr) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long ev = ctr[0]++;
    int parity = (int)(ev & 1ull);
    Stream r(seed, 0xFFFFFFE0u, (uint32_t)ev, (uint32_t)(ev >> 32));
    for (int g = 0; g < nLadders; ++g) {
        int s0 = ladderStart[g], s1 = ladderStart[g + 1];
        for (int k = s0 + parity; k + 1 < s1; k += 2) {
            int ri = ladder[k], rj = ladder[k + 1];
            double Ti = A[ri].temper, Tj = A[rj].temper;
            double Ei = A[ri].ctl->energy, Ej = A[rj].ctl->energy;
            const double* bi = A[ri].s.box;
            const double* bj = A[rj].s.box;
            double Vi = bi[0] * bi[1] * bi[2], Vj = bj[0] * bj[1] * bj[2];
            // canonical and isobaric terms of movecreator.cpp:721-727
            double delta = (1.0 / Ti - 1.0 / Tj) * (Ei - Ej);
            delta += (A[ri].press / Ti - A[rj].press / Tj) * (Vi - Vj);
            delta += gcExchangeTerm(A[ri], A[rj], Ti, Tj);     // grand-canonical term (movecreator.cpp:728-734)
            double u = r.next();
            ctr[1 + 2 * k] += 1ull;
            if (delta >= 0.0 || exp(delta) > u) {
                A[ri].temper = Tj;
                A[rj].temper = Ti;
                if (AC) { AC[ri].temper = Tj; AC[rj].temper = Ti; }   // the chain phase's records
                ladder[k] = rj;
                ladder[k + 1] = ri;
                ctr[2 + 2 * k] += 1ull;
            }
        }
    }
}


// ---- grand-canonical moves -----------------------------------------------------------------
// MoveCreator::muVTMove (scOOP/mc/movecreator.cpp:797-924), one move every nGrandCanon sweeps
// (updater.cpp:164-179).  A species is drawn among the grand-canonical ones (getRandomMuVTType,
// :926-945).  With probability 1/2 a particle of it is inserted at a uniform position
// (Cuboid::randomPos, geometry.h:130-132) with a uniform axis and patch direction
// (Vector::randomUnitSphere, Vector.h:190-205) put through Particle::init (particle.cpp:3-79),
// and kept if V/(N+1) exp(chemPot - E/T) > u; otherwise a uniformly chosen particle of it is
// removed if N/V exp(E/T - chemPot) > u (nothing to remove: rejected).  E is the particle's
// energy against every other particle with an empty conlist (TotalE::mol2others,
// totalenergycalculator.h:211-228).  An insertion takes slot first[m+1], the end of the
// species' block (ParticleVector::insertMolecule, Conf.h:267-275); a removal closes its slot
// (removeMolecule, :277-289): the particles behind move by one slot, so the particle order is
// the reference's.  Only single particles sit behind the first species (Context::setup), so no
// bond partner index changes.
//
// One CTA per system: thread 0 draws the move, every thread sums a strided share of E (fixed
// reduction order), the CTA moves the tail, and the new count goes into the system's device
// arguments (and the chain phase's), which the next sweep's kernels read.

constexpr int kGcThreads = 256;

struct GcSpecies {
    int molType;          // molecule type (index of ParticleVector::first)
    int ctype;            // compact type of its particle
    double chemPot;       // log(activity Nav 1e-24), inicializer.cpp:1094
};

struct GcDev {
    int nSpecies;
    int molTypeCount;
    int cap;              // particle slots of the state arrays (the host keeps one free per move)
    int pad_;
    double chainprob;     // chain moves per particle move: the chain phase's share follows N
    GcSpecies sp[kMaxGrandSpecies];
    int first[MAXMT + 1];                             // ParticleVector::first, kept current
    unsigned long long ctr[kMaxGrandSpecies][5];      // steps, insert acc / rej, delete acc / rej
    double countSum[kMaxGrandSpecies];                // Statistics::grand muVtAverageParticles
};

// The grand-canonical term of the exchange criterion (movecreator.cpp:728-734): for every
// species, (1/T_i - 1/T_j) chemPot T_i (N_i - N_j), chemPot and the species those of system
// i (the replicas share one topology), the counts each system's own.
__device__ double gcExchangeTerm(const SweepArgs& ai, const SweepArgs& aj, double Ti, double Tj) {
    if (!ai.gc || !aj.gc) return 0.0;
    const GcDev& gi = *ai.gc;
    const GcDev& gj = *aj.gc;
    double t = 0.0;
    for (int k = 0; k < gi.nSpecies; ++k) {
        const int m = gi.sp[k].molType;
        const double ni = gi.first[m + 1] - gi.first[m], nj = gj.first[m + 1] - gj.first[m];
        t += (1.0 / Ti - 1.0 / Tj) * gi.sp[k].chemPot * Ti * (ni - nj);
    }
    return t;
}

// Vector::rotate(axis, cos, sin) (Vector.h:133-157): v turned about a unit axis.
__device__ __forceinline__ void gcRotate(double (&v)[3], const double (&ax)[3], double c, double s) {
    const double qw = c, qx = ax[0] * s, qy = ax[1] * s, qz = ax[2] * s;
    const double t2 = qw * qx, t3 = qw * qy, t4 = qw * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
                 t9 = qy * qz, t10 = -qz * qz;
    const double x = v[0], y = v[1], z = v[2];
    v[0] = 2.0 * ((t8 + t10) * x + (t6 - t4) * y + (t3 + t7) * z) + x;
    v[1] = 2.0 * ((t4 + t6) * x + (t5 + t10) * y + (t9 - t2) * z) + y;
    v[2] = 2.0 * ((t7 - t3) * x + (t2 + t9) * y + (t5 + t8) * z) + z;
}
__device__ __forceinline__ void gcNormalise(double (&v)[3]) {
    double t = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (t != 0.0) { t = 1.0 / t; v[0] *= t; v[1] *= t; v[2] *= t; }
}
__device__ __forceinline__ void gcOrthogonalise(double (&v)[3], const double (&b)[3]) {
    const double dp = v[0] * b[0] + v[1] * b[1] + v[2] * b[2];
    v[0] -= dp * b[0]; v[1] -= dp * b[1]; v[2] -= dp * b[2];
}
__device__ __forceinline__ void gcCopy(double (&d)[3], const double (&s)[3]) { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; }

// Particle::init (particle.cpp:3-79) for type g: the axis is normalised, P.pd[0] made a unit
// vector orthogonal to it, and the patch sides (second patch, chiral axes) follow from them.
__device__ void gcInitParticle(const TypeInit& g, double (&dir)[3], PatchSet& P) {
    const int geo = g.geo;
    if (geo == SCA || geo == SCN) return;
    gcNormalise(dir);
    gcOrthogonalise(P.pd[0], dir);
    gcNormalise(P.pd[0]);
    if (geo == PSC || geo == CPSC || geo == TPSC || geo == TCPSC) {
        gcCopy(P.ps[0], P.pd[0]); gcRotate(P.ps[0], dir, g.pcos0, g.psin0);
        gcCopy(P.ps[1], P.pd[0]); gcRotate(P.ps[1], dir, g.pcos0, -1.0 * g.psin0);
    }
    if (isTwoPatch(geo)) {
        gcCopy(P.pd[1], P.pd[0]);
        gcRotate(P.pd[1], dir, g.csec, g.ssec);
        gcOrthogonalise(P.pd[1], dir);
        gcNormalise(P.pd[1]);
    }
    if (geo == TPSC || geo == TCPSC) {
        gcCopy(P.ps[2], P.pd[1]); gcRotate(P.ps[2], dir, g.pcos2, g.psin2);
        gcCopy(P.ps[3], P.pd[1]); gcRotate(P.ps[3], dir, g.pcos2, -1.0 * g.psin2);
    }
    if (isChiral(geo)) {
        gcCopy(P.ch[0], dir); gcRotate(P.ch[0], P.pd[0], g.chcos, g.chsin);
        gcCopy(P.ps[0], P.pd[0]); gcRotate(P.ps[0], P.ch[0], g.pcos0, g.psin0);
        gcCopy(P.ps[1], P.pd[0]); gcRotate(P.ps[1], P.ch[0], g.pcos0, -1.0 * g.psin0);
    }
    if (geo == TCHPSC || geo == TCHCPSC) {
        gcCopy(P.ch[1], dir); gcRotate(P.ch[1], P.pd[1], g.chcos, g.chsin);
        gcCopy(P.ps[2], P.pd[1]); gcRotate(P.ps[2], P.ch[1], g.pcos2, g.psin2);
        gcCopy(P.ps[3], P.pd[1]); gcRotate(P.ps[3], P.ch[1], g.pcos2, -1.0 * g.psin2);
    }
}

// Moves particle slot `from` to slot `to` (the state arrays and the molecule record, whose
// first-particle field is the slot itself for the single particles that move).
struct GcSlot {
    double4_32a pos, dir;
    PatchSet patch;
    int4 mol;
};
__device__ __forceinline__ void gcLoad(const DevState& s, int i, GcSlot& v) {
    v.pos = s.pos[i];
    v.dir = s.dir[i];
    v.patch = s.patch[i];
    v.mol = s.mol[i];
}
__device__ __forceinline__ void gcStore(const DevState& s, int i, const GcSlot& v) {
    s.pos[i] = v.pos;
    s.dir[i] = v.dir;
    s.patch[i] = v.patch;
    int4 m = v.mol;
    m.w = i;
    s.mol[i] = m;
}

__global__ void __launch_bounds__(kGcThreads) kGrandCanon(SweepArgs* A, SweepArgs* AC) {
    SweepArgs& a = A[blockIdx.y];
    if (!a.gc || blockIdx.x != 0) return;
    GcDev& g = *a.gc;
    Control& ctl = *a.ctl;
    __shared__ int sSpecies, sInsert, sSlot, sCount, sSkip, sAccept;
    __shared__ double sU, sPos[3], sDir[3];
    __shared__ PatchSet sPatch;
    __shared__ double sWarp[kGcThreads / 32];
    const int n = a.s.n;
    if (threadIdx.x == 0) {
        Stream r(a.seed ^ 0xA0761D6478BD642Full, 0xFFFFFFE8u, (uint32_t)ctl.sweep, (uint32_t)(ctl.sweep >> 32));
        const int k = min((int)(r.next() * g.nSpecies), g.nSpecies - 1);
        const GcSpecies& sp = g.sp[k];
        const int count = g.first[sp.molType + 1] - g.first[sp.molType];
        sSpecies = k;
        sCount = count;
        sSkip = 0;
        sInsert = r.next() > 0.5 ? 1 : 0;
        if (sInsert) {
            for (int d = 0; d < 3; ++d) sPos[d] = r.next();
            double dir[3], pd[3];
            randomUnitSphere(r, dir[0], dir[1], dir[2]);
            randomUnitSphere(r, pd[0], pd[1], pd[2]);
            PatchSet P;
            for (int q = 0; q < 3; ++q) {
                P.pd[0][q] = pd[q]; P.pd[1][q] = 0.0;
                for (int w = 0; w < 4; ++w) P.ps[w][q] = 0.0;
                P.ch[0][q] = 0.0; P.ch[1][q] = 0.0;
            }
            gcInitParticle(a.tinit[sp.ctype], dir, P);
            for (int d = 0; d < 3; ++d) sDir[d] = dir[d];
            sPatch = P;
            sSlot = g.first[sp.molType + 1];
            if (n >= g.cap) {             // the host keeps a free slot before every move
                atomicOr(a.err, E_GC_FULL);
                sSkip = 2;
            }
        } else if (count == 0) {
            sSkip = 1;                    // nothing to remove (movecreator.cpp:882-886)
        } else {
            sSlot = g.first[sp.molType] + min((int)(r.next() * count), count - 1);
        }
        sU = r.next();
    }
    __syncthreads();
    const int k = sSpecies;
    const GcSpecies& sp = g.sp[k];
    if (sSkip) {
        if (threadIdx.x == 0 && sSkip == 1) {
            g.ctr[k][0] += 1ull;
            g.ctr[k][4] += 1ull;
            g.countSum[k] += (double)sCount;
        }
        return;
    }
    DevCtx c;
    c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = n; c.sqmaxcut = a.t.sqmaxcut;
    const double3 box = mk(a.s.box[0], a.s.box[1], a.s.box[2]);
    const bool insert = sInsert != 0;
    const int slot = sSlot;
    PView me;
    if (insert) {
        me.pos = mk(sPos[0], sPos[1], sPos[2]);
        me.dir = mk(sDir[0], sDir[1], sDir[2]);
        me.patch = &sPatch;
        me.type = sp.ctype;
        me.index = -1;
        me.molType = sp.molType;
    } else {
        const double4_32a p = a.s.pos[slot], d = a.s.dir[slot];
        me.pos = mk(p.x, p.y, p.z);
        me.dir = mk(d.x, d.y, d.z);
        me.patch = &a.s.patch[slot];
        me.type = (int)p.w;
        me.index = slot;
        me.molType = a.s.mol[slot].x;
    }
    const Con con = emptyCon(c);
    double e = 0.0;
    for (int j = threadIdx.x; j < n; j += kGcThreads) {
        if (!insert && j == slot) continue;
        const double4_32a p = a.s.pos[j], d = a.s.dir[j];
        PView b;
        b.pos = mk(p.x, p.y, p.z);
        b.dir = mk(d.x, d.y, d.z);
        b.patch = &a.s.patch[j];
        b.type = (int)p.w;
        b.index = j;
        b.molType = a.s.mol[j].x;
        unsigned bits;
        double dsq;
        e += pairEnergy(c, me, b, con, box, &bits, &dsq);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if ((threadIdx.x & 31) == 0) sWarp[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double E = 0.0;
        for (int w = 0; w < kGcThreads / 32; ++w) E += sWarp[w];
        const double V = box.x * box.y * box.z;
        const int count = sCount;
        bool acc;
        if (insert) acc = (V / (count + 1.0)) * exp(sp.chemPot - E / a.temper) > sU;
        else acc = ((double)count / V) * exp(E / a.temper - sp.chemPot) > sU;
        g.ctr[k][0] += 1ull;
        g.ctr[k][insert ? (acc ? 1 : 2) : (acc ? 3 : 4)] += 1ull;
        g.countSum[k] += (double)(acc ? (insert ? count + 1 : count - 1) : count);
        if (acc) ctl.energy += insert ? E : -1.0 * E;
        sAccept = acc ? 1 : 0;
    }
    __syncthreads();
    if (!sAccept) return;
    GcSlot v;
    if (insert) {
        // the tail [slot, n) moves up by one, highest chunk first: a chunk reads all its slots
        // before any thread writes, and writes only slots the chunks below do not read
        for (int hi = n; hi > slot; hi -= kGcThreads) {
            const int lo = max(slot, hi - kGcThreads);
            const int i = lo + (int)threadIdx.x;
            if (i < hi) gcLoad(a.s, i, v);
            __syncthreads();
            if (i < hi) gcStore(a.s, i + 1, v);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            v.pos = make_double4_32a(sPos[0], sPos[1], sPos[2], (double)sp.ctype);
            v.dir = make_double4_32a(sDir[0], sDir[1], sDir[2], 0.0);
            v.patch = sPatch;
            v.mol = make_int4(sp.molType, 0, 1, slot);
            gcStore(a.s, slot, v);
        }
    } else {
        // the tail (slot, n) moves down by one, lowest chunk first
        for (int lo = slot + 1; lo < n; lo += kGcThreads) {
            const int i = lo + (int)threadIdx.x;
            if (i < n) gcLoad(a.s, i, v);
            __syncthreads();
            if (i < n) gcStore(a.s, i - 1, v);
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        const int dn = insert ? 1 : -1;
        for (int m = sp.molType + 1; m <= g.molTypeCount; ++m) g.first[m] += dn;
        a.s.n = n + dn;
        if (AC) {           // the chain phase: its count, and N chainprob chain moves per sweep
            SweepArgs& ac = AC[blockIdx.y];
            ac.s.n = n + dn;
            if (ac.nChains > 0) ac.chainFrac = g.chainprob * (double)(n + dn) / (double)ac.nChains;
        }
    }
}


// ---- type switching ----------------------------------------------------------------------
// MoveCreator::switchTypeMove (scOOP/mc/movecreator.cpp:233-303): a particle with a switch
// type takes the other type of its pair -- its switch type when unswitched, its molecule's
// type when switched -- and Particle::init re-derives its patch vectors for that type; the
// move is kept under moveTry(E_old, E_new + delta_mu (1 - 2 switched)) (movecreator.h:175-187),
// E the particle against every other with its conlist (oneToAll / oneToAllTrial), delta_mu
// the int the reference reads it into.  A rejected move re-initialises the patch vectors
// for the old type, as the reference does.  The reference makes N switchprob attempts per
// sweep, each on a uniformly chosen switchable particle.
//
// On the GPU the attempts are a checkerboard phase after each sweep's particle moves, over
// the sweep's cell list (every particle is still in its cell: a move that would leave it is
// rejected): one CTA per active cell of a colour, the colours in the sweep's order.  A cell
// makes cnt * rate attempts (rate = switchprob N / switchable particles, the fraction rounded
// at random), each on a uniformly chosen particle of the cell and skipped when that one has
// no switch type, so every switchable particle sees the reference's attempt rate.  The
// energies are full FP64 pair energies against the cell's stencil (reach s: every particle
// within maxcut), reduced in a fixed order.

constexpr int kSwThreads = 128;

struct SwitchShared {
    Stencil st;
    Scan scan;
    PatchSet newP, oldP;         // patch vectors under the new type / re-derived for the old one
    double dirNew[3], dirOld[3];
    double u;
    int target, oldType, newType, switched, dmu, go;
    double redO[kSwThreads / 32], redN[kSwThreads / 32];
    int redP[kSwThreads / 32];
};

__global__ void __launch_bounds__(kSwThreads) kSwitchColour(const SweepArgs* __restrict__ A, int phase) {
    const SweepArgs& a = A[blockIdx.y];
    if (!a.swTab || !(a.switchRate > 0.0)) return;
    const Grid& g = a.g;
    if ((int)blockIdx.x >= g.nactive || phase >= g.ncolours) return;
    int cx, cy, cz;
    decodeActive(g, a.ctl->perm[phase], blockIdx.x, cx, cy, cz);
    const int cell = (cz * g.nc[1] + cy) * g.nc[0] + cx;
    const int cnt = a.cellCount[cell];
    if (cnt == 0) return;
    __shared__ SwitchShared sh;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    stageStencil<kSwThreads>(a, cx, cy, cz, sh.st, sh.scan);
    const Control& ctl = *a.ctl;
    const uint32_t sk = (uint32_t)ctl.sweep ^ ((uint32_t)(ctl.sweep >> 32) << 20);
    const uint64_t seed = a.seed ^ 0x5851F42D4C957F2Dull;
    int nAtt;
    {
        Stream r(seed, (uint32_t)cell, 0xFFFFFFFFu, sk);
        const double want = cnt * a.switchRate;
        nAtt = (int)want;
        if (r.next() < want - nAtt) ++nAtt;
    }
    DevCtx c;
    c.params = a.t.params; c.mols = a.t.mols; c.ntypes = a.t.ntypes; c.n = a.s.n; c.sqmaxcut = a.t.sqmaxcut;
    const double3 box = mk(a.s.box[0], a.s.box[1], a.s.box[2]);
    double dE = 0.0;
    unsigned long long nAcc = 0, nRej = 0;
    for (int m = 0; m < nAtt; ++m) {
        if (tid == 0) {
            Stream r(seed, (uint32_t)cell, (uint32_t)m, sk);
            const int slot = min((int)(r.next() * cnt), cnt - 1);
            const int t = a.cellIdx[a.cellStart[cell] + slot];
            const int4 mol = a.s.mol[t];
            const int4 sw = mol.y < MAXCHL ? a.swTab[mol.x * MAXCHL + mol.y] : make_int4(-1, -1, 0, 0);
            sh.go = 0;
            if (sw.y >= 0) {
                const double4_32a d = a.s.dir[t];
                const int switched = d.w != 0.0 ? 1 : 0;
                sh.go = 1;
                sh.target = t;
                sh.switched = switched;
                sh.oldType = (int)a.s.pos[t].w;
                sh.newType = switched ? sw.x : sw.y;
                sh.dmu = sw.z;
                double dir[3] = {d.x, d.y, d.z};
                PatchSet P = a.s.patch[t];
                gcInitParticle(a.tinit[sh.newType], dir, P);
                for (int q = 0; q < 3; ++q) sh.dirNew[q] = dir[q];
                sh.newP = P;
                gcInitParticle(a.tinit[sh.oldType], dir, P);     // the reject path: init again, old type
                for (int q = 0; q < 3; ++q) sh.dirOld[q] = dir[q];
                sh.oldP = P;
                sh.u = r.next();
            }
        }
        __syncthreads();
        if (sh.go) {
            const int t = sh.target;
            const double4_32a p = a.s.pos[t], d = a.s.dir[t];
            const int4 mol = a.s.mol[t];
            PView vo, vn;
            vo.pos = vn.pos = mk(p.x, p.y, p.z);
            vo.dir = mk(d.x, d.y, d.z);
            vn.dir = mk(sh.dirNew[0], sh.dirNew[1], sh.dirNew[2]);
            vo.patch = &a.s.patch[t];
            vn.patch = &sh.newP;
            vo.type = sh.oldType;
            vn.type = sh.newType;
            vo.index = vn.index = t;
            vo.molType = vn.molType = mol.x;
            const Con con = makeCon(c, t, mol);
            double eo = 0.0, en = 0.0;
            int partners = 0;
            for (int k = tid; k < sh.st.nCand; k += kSwThreads) {
                int lo = 0, hi = sh.st.nNb;          // nbOff[lo] <= k < nbOff[hi]
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (sh.st.nbOff[mid] <= k) lo = mid;
                    else hi = mid;
                }
                const int j = a.cellIdx[a.cellStart[sh.st.nbCell[lo]] + (k - sh.st.nbOff[lo])];
                if (j == t) continue;
                const double4_32a q = a.s.pos[j], e = a.s.dir[j];
                PView b;
                b.pos = mk(q.x, q.y, q.z);
                b.dir = mk(e.x, e.y, e.z);
                b.patch = &a.s.patch[j];
                b.type = (int)q.w;
                b.index = j;
                b.molType = a.s.mol[j].x;
                unsigned bits;
                double dsq;
                eo += pairEnergy(c, vo, b, con, box, &bits, &dsq);
                en += pairEnergy(c, vn, b, con, box, &bits, &dsq);
                partners += (j == con.idx[0]) + (j == con.idx[1]) + (j == con.idx[2]) + (j == con.idx[3]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                eo += __shfl_down_sync(0xffffffffu, eo, o);
                en += __shfl_down_sync(0xffffffffu, en, o);
                partners += __shfl_down_sync(0xffffffffu, partners, o);
            }
            if (lane == 0) { sh.redO[warp] = eo; sh.redN[warp] = en; sh.redP[warp] = partners; }
            __syncthreads();
            if (tid == 0) {
                double Eo = 0.0, En = 0.0;
                int found = 0;
                for (int w = 0; w < kSwThreads / 32; ++w) { Eo += sh.redO[w]; En += sh.redN[w]; found += sh.redP[w]; }
                const int want = (con.idx[0] >= 0) + (con.idx[1] >= 0) + (con.idx[2] >= 0) + (con.idx[3] >= 0);
                if (found < want) {             // a bonded partner outside the stencil: no decision
                    atomicOr(a.err, E_PARTNER_FAR);
                } else {
                    const int pmone = 1 - 2 * sh.switched;
                    const double enew = En + (double)(sh.dmu * pmone);
                    const bool acc = (enew <= Eo) || (exp(-1.0 * (enew - Eo) / a.temper) > sh.u);
                    if (acc) {
                        a.s.pos[t] = make_double4_32a(p.x, p.y, p.z, (double)sh.newType);
                        a.s.dir[t] = make_double4_32a(sh.dirNew[0], sh.dirNew[1], sh.dirNew[2],
                                                      (double)(sh.switched + pmone));
                        a.s.patch[t] = sh.newP;
                        dE += En - Eo;
                        ++nAcc;
                    } else {
                        a.s.dir[t] = make_double4_32a(sh.dirOld[0], sh.dirOld[1], sh.dirOld[2], d.w);
                        a.s.patch[t] = sh.oldP;
                        ++nRej;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        a.cellDE[cell] += dE;
        if (nAcc) atomicAdd(&a.counters[C_ACC_SW], nAcc);
        if (nRej) atomicAdd(&a.counters[C_REJ_SW], nRej);
    }
}

}  // namespace

// Device state of the move loop of one system.
struct SweepEngine {
    Grid g{};
    Control* ctl = nullptr;
    int *cellStart = nullptr, *cellCount = nullptr, *cellCursor = nullptr, *cellIdx = nullptr, *cellOf = nullptr;
    float4* cellPosF = nullptr;
    float4* cellDirF = nullptr;
    float4* cellPatF = nullptr;
    double* cellDE = nullptr;
    unsigned* cellDone = nullptr;
    double* partial = nullptr;
    unsigned long long* counters = nullptr;
    int* err = nullptr;
    int ncellsAlloc = 0;
    std::vector<void*> allocs;
    bool energyKnown = false;
    unsigned long long* typeCtr = nullptr;        // per-type acceptance of the run (SweepArgs::typeCtr)
    GcDev* gc = nullptr;          // grand-canonical record (kGrandCanon)
    TypeInit* tinit = nullptr;    // Particle::init parameters per compact type
    sc_run_params runParams{};    // the parameters the system's arguments were filled from
    bool gcOn = false;            // this run makes grand-canonical moves
    int slots = 0;                // particle slots of the per-particle buffers below and of the chain phase
    uint64_t seed = ~0ull;
    int stencil = 0;
    double margin = 0.0;
    SweepArgs args{};
    // chain moves: the chain grid's particle cell list, the chains binned by centre
    struct Chains {
        bool on = false;
        Grid g{};
        Control* ctl = nullptr;
        int *cellStart = nullptr, *cellCount = nullptr, *cellCursor = nullptr, *cellIdx = nullptr, *cellOf = nullptr;
        int* slotOf = nullptr;
        float4* cellPosF = nullptr;
        double* cellDE = nullptr;
        unsigned* cellDone = nullptr;
        int2* chains = nullptr;
        int nChains = 0;
        int *chStart = nullptr, *chCount = nullptr, *chIdx = nullptr;
        int ncellsAlloc = 0;
        double R = 0.0;
        SweepArgs args{};
    } ch;
};

// A set of systems moved together: one launch sequence per sweep, blockIdx.y = system.
struct Batch {
    std::vector<Context*> sys;
    std::vector<SweepArgs> hArgs;
    SweepArgs* dArgs = nullptr;
    int nArgsAlloc = 0;
    int maxN = 0, maxCells = 0, maxActive = 0, maxColours = 0;
    // chain phase (every system of the batch holds chains, or none does)
    bool chains = false;
    bool wl = false;          // a system carries a Wang-Landau bias
    bool switching = false;   // a system makes type switch moves
    std::vector<SweepArgs> hArgsC;
    SweepArgs* dArgsC = nullptr;
    int nArgsCAlloc = 0;
    int maxCellsC = 0, maxActiveC = 0, maxColoursC = 0;
    cudaStream_t stream = nullptr;
    int device = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> evPhase;     // time_phases: start / end of each sweep's move launches
    cudaGraphExec_t graph = nullptr;
    int graphDims[16] = {0};   // launch shape the graph was captured with
    long graphLaunches = 0, graphPhaseLaunches = 0;
    // parallel tempering
    int* dLadder = nullptr;
    int* dLadderStart = nullptr;
    int nLadders = 0;
    unsigned long long* dExCtr = nullptr;
    std::vector<void*> allocs;

    ~Batch() {
        DeviceScope dev(device);
        for (void* p : allocs) cudaFree(p);
        for (cudaEvent_t e : {ev0, ev1})
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : evPhase) cudaEventDestroy(e);
        if (graph) cudaGraphExecDestroy(graph);
    }
    int alloc(void** p, size_t bytes) {
        cudaError_t r = cudaMalloc(p, bytes ? bytes : 16);
        if (r != cudaSuccess) return cudaFail(r, "cudaMalloc (batch)");
        allocs.push_back(*p);
        return SC_OK;
    }
};

static int engineAlloc(SweepEngine* e, void** p, size_t bytes) {
    cudaError_t r = cudaMalloc(p, bytes ? bytes : 16);
    if (r != cudaSuccess) return cudaFail(r, "cudaMalloc (sweep)");
    e->allocs.push_back(*p);
    return SC_OK;
}

// Cell grid for a box.  With reach s the cells are >= maxcut*(1+margin)/s wide and the
// count per dimension is a multiple of the colour period s+1 (and > 2s, so that the
// stencil cells are distinct); dimensions too small for that fall back to reach 1 with
// an even count (or 1 / 2 cells).
static Grid makeGrid(const double* box, double maxcut, double margin, int sReq) {
    Grid g{};
    g.maxcut = maxcut;
    for (int d = 0; d < 3; ++d) {
        bool ok = false;
        if (sReq >= 2) {
            int p = sReq + 1;
            int nc = (int)std::floor(box[d] / (maxcut * (1.0 + margin) / sReq));
            nc -= nc % p;
            if (nc > 2 * sReq) { g.nc[d] = nc; g.p[d] = p; g.s[d] = sReq; ok = true; }
        }
        if (!ok) {
            int nc = (int)std::floor(box[d] / (maxcut * (1.0 + margin)));
            if (nc < 1) nc = 1;
            if (nc >= 3 && (nc & 1)) nc -= 1;
            g.nc[d] = nc;
            g.p[d] = nc >= 2 ? 2 : 1;
            g.s[d] = 1;
        }
    }
    g.ncells = g.nc[0] * g.nc[1] * g.nc[2];
    g.nactive = (g.nc[0] / g.p[0]) * (g.nc[1] / g.p[1]) * (g.nc[2] / g.p[2]);
    g.ncolours = g.p[0] * g.p[1] * g.p[2];
    return g;
}

// Stencil reach: 2 (cells of maxcut/2, 27 colours) when the box holds at least 6 such
// cells per dimension, else 1.
static int chooseStencil(const double* box, double maxcut, int requested) {
    if (requested >= 1 && requested <= 3) return requested;
    double lim = std::min(box[0], std::min(box[1], box[2]));
    return lim / (maxcut / 2.0) >= 6.0 ? 2 : 1;
}

void destroyEngine(Context* c) {
    if (c->batch) {
        delete c->batch;
        c->batch = nullptr;
    }
    SweepEngine* e = c->engine;
    if (!e) return;
    DeviceScope dev(c->device);
    for (void* p : e->allocs) cudaFree(p);
    delete e;
    c->engine = nullptr;
}

static void engineFree(SweepEngine* e, void** p) {
    if (!*p) return;
    cudaFree(*p);
    e->allocs.erase(std::find(e->allocs.begin(), e->allocs.end(), *p));
    *p = nullptr;
}

// Per-particle buffers of the cell lists (and of the chain phase's, once it exists) for
// `slots` particles; their contents are rebuilt every sweep.
static int particleBuffers(SweepEngine* e, int slots) {
    int rc;
    for (void** p : {(void**)&e->cellIdx, (void**)&e->cellPosF, (void**)&e->cellDirF, (void**)&e->cellPatF,
                     (void**)&e->cellOf})
        engineFree(e, p);
    if ((rc = engineAlloc(e, (void**)&e->cellIdx, sizeof(int) * slots))) return rc;
    if ((rc = engineAlloc(e, (void**)&e->cellPosF, sizeof(float4) * slots))) return rc;
    if ((rc = engineAlloc(e, (void**)&e->cellDirF, sizeof(float4) * slots))) return rc;
    if ((rc = engineAlloc(e, (void**)&e->cellPatF, sizeof(float4) * slots))) return rc;
    if ((rc = engineAlloc(e, (void**)&e->cellOf, sizeof(int) * slots))) return rc;
    SweepEngine::Chains& C = e->ch;
    if (C.ctl) {
        for (void** p : {(void**)&C.cellIdx, (void**)&C.cellOf, (void**)&C.slotOf, (void**)&C.cellPosF}) engineFree(e, p);
        if ((rc = engineAlloc(e, (void**)&C.cellIdx, sizeof(int) * slots))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellOf, sizeof(int) * slots))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.slotOf, sizeof(int) * slots))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellPosF, sizeof(float4) * slots))) return rc;
    }
    e->slots = slots;
    return SC_OK;
}

static int ensureGrid(Context* c, SweepEngine* e, const double* box) {
    Grid g = makeGrid(box, c->topo.maxcut, e->margin, e->stencil);
    if (g.ncolours > kMaxColours) return fail(SC_ERR_RANGE, "too many colour classes");
    if (g.ncells > e->ncellsAlloc) {
        for (void** p : {(void**)&e->cellStart, (void**)&e->cellCount, (void**)&e->cellCursor, (void**)&e->cellDE,
                         (void**)&e->partial, (void**)&e->cellDone}) {
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
        if ((rc = engineAlloc(e, (void**)&e->partial, sizeof(double) * n))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->cellDone, sizeof(unsigned) * n))) return rc;
        cudaMemset(e->cellDE, 0, sizeof(double) * n);
        cudaMemset(e->cellDone, 0, sizeof(unsigned) * n);
        e->ncellsAlloc = n;
    }
    e->g = g;
    return SC_OK;
}

// Chain displacement length of molecule type m: the adapted step (sc_adjust_steps), scaled as
// the run's chainmmx scales the options value, else the run's chainmmx.
static double chainStep(const Context* c, int m, const sc_run_params& p) {
    if (m < Context::kMaxChainSteps && c->chainAdapted[m] > 0.0 && c->opts.chainmmx > 0.0)
        return c->chainAdapted[m] * (p.chainmmx / c->opts.chainmmx);
    return p.chainmmx;
}

static void fillArgs(Context* c, SweepEngine* e, const sc_run_params& p) {
    SweepArgs& a = e->args;
    std::memset(&a, 0, sizeof a);
    a.s = c->d;
    a.t = c->tables;
    a.g = e->g;
    a.ctl = e->ctl;
    a.cellStart = e->cellStart; a.cellCount = e->cellCount; a.cellCursor = e->cellCursor;
    a.cellIdx = e->cellIdx; a.cellPosF = e->cellPosF; a.cellOf = e->cellOf; a.cellDE = e->cellDE;
    a.cellDirF = e->cellDirF; a.cellPatF = e->cellPatF;
    a.cellDone = e->cellDone;
    a.partial = e->partial;
    a.counters = e->counters; a.err = e->err;
    a.seed = p.seed;
    a.temper = p.temper;
    a.press = p.press;
    a.rotAngle = p.rot_angle;
    a.edgeMx = p.edge_mx;
    a.ptype = p.ptype;
    a.pairMoves = (p.variant & 2) ? 1 : 0;
    for (size_t k = 0; k < c->usedTypes.size() && k < (size_t)MAX_DEV_TYPES; ++k) {
        int t = c->usedTypes[k];
        // per-type displacement (sim.h:368-373); the run's transmx replaces the options value
        double base = c->opts.transmx;
        double perType = c->opts.trans_type[t];
        a.trans[k] = (base > 0 && perType != base) ? perType * (p.transmx / base) : p.transmx;
        a.geo[k] = c->topo.ia[t][t].geotype[0];
        a.volW[k] = c->topo.ia[t][t].volume;
    }
    if (p.delayed && c->surrogate) {
        a.mlp = surrogatePacked(c->surrogate);
        a.rcutS = surrogateCutoff(c->surrogate);
    }
    a.wl = wlDevice(c);
    a.flowSpin = p.flow_wait_polls > 0 ? p.flow_wait_polls : kFlowSpin;
    a.typeCtr = e->typeCtr;
    a.coneAngle = c->opts.coneAngle;
    for (int m = 0; m < kMaxChainTypes; ++m) a.chainMxType[m] = chainStep(c, m, p);
    a.gc = e->gcOn ? e->gc : nullptr;
    a.tinit = e->tinit;
    // type switching: N switchprob attempts per sweep spread over the switchable particles
    // (each cell makes cnt * rate attempts on random particles of the cell)
    a.swTab = nullptr;
    a.switchRate = 0.0;
    if (p.switchprob > 0.0 && c->anySwitch) {
        long nsw = 0;
        for (const int4& mi : c->molInfo)
            if (mi.y < MAXCHL && c->switchTab[(size_t)mi.x * MAXCHL + mi.y].y >= 0) ++nsw;
        if (nsw > 0) {
            a.swTab = c->dSwitch;
            a.switchRate = p.switchprob * (double)c->d.n / (double)nsw;
        }
    }
}

// Chain phase of one system: chains (molecules of more than one particle), the bound R of
// their half-extent, the chain grid (cells >= (maxcut + 2 (R + displacement)) / 2) and its
// arguments.  Off when chainprob is 0 or the system holds no chains.
static int prepareChains(Context* c, SweepEngine* e, const sc_run_params& p, const double* box) {
    SweepEngine::Chains& C = e->ch;
    C.on = false;
    std::vector<int2> chains;
    for (size_t i = 0; i < c->molInfo.size(); ++i)
        if (c->molInfo[i].y == 0 && c->molInfo[i].z > 1) chains.push_back(make_int2((int)i, c->molInfo[i].z));
    if (!(p.chainprob > 0) || chains.empty()) return SC_OK;
    for (const int2& ch : chains)
        if (ch.y > kMaxChain) return fail(SC_ERR_RANGE, "a chain holds more than 20 particles (MAXCHL)");
    int rc;
    const int n = c->d.n;
    if (!C.ctl) {
        if ((rc = engineAlloc(e, (void**)&C.ctl, sizeof(Control)))) return rc;
        cudaMemset(C.ctl, 0, sizeof(Control));
        const int slots = std::max(e->slots, 1);
        if ((rc = engineAlloc(e, (void**)&C.cellIdx, sizeof(int) * slots))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellOf, sizeof(int) * slots))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.slotOf, sizeof(int) * slots))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellPosF, sizeof(float4) * slots))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.chains, sizeof(int2) * chains.size()))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.chIdx, sizeof(int) * chains.size()))) return rc;
        cudaMemcpy(C.chains, chains.data(), sizeof(int2) * chains.size(), cudaMemcpyHostToDevice);
        C.nChains = (int)chains.size();
    }
    if (e->seed != p.seed) {
        unsigned long long zero = 0;
        cudaMemcpy(&C.ctl->sweep, &zero, sizeof zero, cudaMemcpyHostToDevice);
    }
    // half-extent bound from the current configuration, with room to stretch
    unsigned* dMax = nullptr;
    if ((rc = engineAlloc(e, (void**)&dMax, sizeof(unsigned)))) return rc;
    cudaMemset(dMax, 0, sizeof(unsigned));
    kChainExtent<<<(C.nChains + 127) / 128, 128, 0, c->stream>>>(e->args, C.chains, C.nChains, dMax);
    unsigned bits = 0;
    cudaError_t r = cudaMemcpyAsync(&bits, dMax, sizeof bits, cudaMemcpyDeviceToHost, c->stream);
    if (r == cudaSuccess) r = cudaStreamSynchronize(c->stream);
    cudaFree(dMax);
    e->allocs.erase(std::find(e->allocs.begin(), e->allocs.end(), (void*)dMax));
    if (r != cudaSuccess) return cudaFail(r, "chain extent");
    float ext;
    std::memcpy(&ext, &bits, sizeof ext);
    C.R = std::max(1.2 * ext, ext + 0.5);
    double step = p.chainmmx;            // the longest chain displacement of any molecule type
    for (int m = 0; m < kMaxChainTypes; ++m) step = std::max(step, chainStep(c, m, p));
    Grid g = makeGrid(box, c->topo.maxcut + 2.0 * (C.R + step), e->margin, 2);
    if (g.ncolours > kMaxColours) return fail(SC_ERR_RANGE, "too many colour classes (chain grid)");
    g.maxcut = c->topo.maxcut + 2.0 * (C.R + step);
    if (g.ncells > C.ncellsAlloc) {
        for (void** q : {(void**)&C.cellStart, (void**)&C.cellCount, (void**)&C.cellCursor, (void**)&C.cellDE,
                         (void**)&C.chStart, (void**)&C.chCount, (void**)&C.cellDone}) {
            if (*q) {
                cudaFree(*q);
                e->allocs.erase(std::find(e->allocs.begin(), e->allocs.end(), *q));
                *q = nullptr;
            }
        }
        int m = g.ncells;
        if ((rc = engineAlloc(e, (void**)&C.cellStart, sizeof(int) * m))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellCount, sizeof(int) * m))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellCursor, sizeof(int) * m))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellDE, sizeof(double) * m))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.chStart, sizeof(int) * m))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.chCount, sizeof(int) * m))) return rc;
        if ((rc = engineAlloc(e, (void**)&C.cellDone, sizeof(unsigned) * m))) return rc;
        cudaMemset(C.cellDE, 0, sizeof(double) * m);
        cudaMemset(C.cellDone, 0, sizeof(unsigned) * m);
        C.ncellsAlloc = m;
    }
    C.g = g;
    SweepArgs& a = C.args;
    a = e->args;
    a.g = g;
    a.ctl = C.ctl;
    a.cellStart = C.cellStart; a.cellCount = C.cellCount; a.cellCursor = C.cellCursor; a.cellIdx = C.cellIdx;
    a.cellOf = C.cellOf; a.cellPosF = C.cellPosF; a.cellDE = C.cellDE;
    a.cellDone = C.cellDone;
    a.slotOf = C.slotOf;
    a.cellDirF = a.cellPatF = nullptr;
    a.mlp = nullptr;
    a.seed = p.seed ^ 0x6A09E667F3BCC909ull;
    a.wl = nullptr;
    a.energyAcc = &e->ctl->energy;
    a.chains = C.chains;
    a.nChains = C.nChains;
    a.chainCellStart = C.chStart; a.chainCellCount = C.chCount; a.chainCellIdx = C.chIdx;
    a.chainMx = p.chainmmx;
    a.chainAngle = p.chain_angle;
    a.chainFrac = p.chainprob * (double)n / (double)C.nChains;   // N * chainprob chain moves per sweep
    a.chainR = C.R;
    C.on = true;
    // volume moves must leave the chain cells wide enough as well
    for (int d = 0; d < 3; ++d) e->args.boxMinChain[d] = g.nc[d] * g.maxcut / g.s[d];
    a.boxMinChain[0] = a.boxMinChain[1] = a.boxMinChain[2] = 0.0;
    return SC_OK;
}

// Grand-canonical record of a run: the species with what Particle::init needs of their type,
// ParticleVector::first, the capacity, zeroed counters.
static int prepareGrand(Context* c, SweepEngine* e, const sc_run_params& p) {
    e->gcOn = p.grand_every > 0 && !c->grand.empty();
    if (!e->gcOn) return SC_OK;
    if (c->conf.molTypeCount > MAXMT) return fail(SC_ERR_RANGE, "more than 100 molecule types (MAXMT)");
    int rc;
    if (!e->gc && (rc = engineAlloc(e, (void**)&e->gc, sizeof(GcDev)))) return rc;
    GcDev h;
    std::memset(&h, 0, sizeof h);
    h.nSpecies = (int)c->grand.size();
    h.molTypeCount = c->conf.molTypeCount;
    h.cap = c->cap;
    h.chainprob = p.chainprob;
    for (int k = 0; k < h.nSpecies; ++k) {
        const Context::Grand& g = c->grand[k];
        GcSpecies& sp = h.sp[k];
        sp.molType = g.molType;
        sp.ctype = c->compactOf[g.type];
        sp.chemPot = g.chemPot;
    }
    for (int m = 0; m <= h.molTypeCount; ++m) h.first[m] = c->conf.first[m];
    cudaError_t r = cudaMemcpy(e->gc, &h, sizeof h, cudaMemcpyHostToDevice);
    if (r != cudaSuccess) return cudaFail(r, "upload grand-canonical record");
    return SC_OK;
}

// After a run with grand-canonical moves: the device's count, ParticleVector::first and
// counters back on the host, and the host particle vector brought to the device's.
static int finishGrand(Context* c, const SweepArgs* dArgs) {
    SweepEngine* e = c->engine;
    if (!e || !e->gcOn) return SC_OK;
    GcDev h;
    SweepArgs cur;
    cudaError_t r = cudaMemcpy(&h, e->gc, sizeof h, cudaMemcpyDeviceToHost);
    if (r == cudaSuccess) r = cudaMemcpy(&cur, dArgs, sizeof cur, cudaMemcpyDeviceToHost);
    if (r != cudaSuccess) return cudaFail(r, "grand-canonical record");
    for (int k = 0; k < h.nSpecies && k < (int)c->grand.size(); ++k) {
        Context::Grand& g = c->grand[k];
        g.steps += (long)h.ctr[k][0];
        g.insAcc += (long)h.ctr[k][1]; g.insRej += (long)h.ctr[k][2];
        g.delAcc += (long)h.ctr[k][3]; g.delRej += (long)h.ctr[k][4];
        g.countSum += h.countSum[k];
    }
    const int n = cur.s.n;
    c->conf.first.assign(h.first, h.first + h.molTypeCount + 1);
    c->conf.p.resize((size_t)n);
    for (int m = 0; m < h.molTypeCount; ++m)
        for (int i = h.first[m]; i < h.first[m + 1] && i < n; ++i) c->conf.p[i].molType = m;
    c->d.n = n;
    e->args.s.n = n;
    e->ch.args.s.n = n;
    c->devNewer = true;
    int rc = c->downloadState();       // positions, axes, patches, types
    c->rebuildMolInfo();
    return rc;
}

// A grand-canonical system whose free slots ran out: larger state arrays and per-particle
// buffers, and the arguments (with the device's count) uploaded again.
// The device copy of a batch's arguments runs ahead of the host's during a run: replica
// exchange swaps temperatures, grand-canonical moves change the particle count (and the chain
// phase's share of moves).  Brings the host copies (and every context's count) up to it, so
// that an upload keeps them (the stream is synchronised).
static int syncDeviceArgs(Batch& b) {
    const int ns = (int)b.sys.size();
    std::vector<SweepArgs> cur(ns), curC;
    cudaError_t r = cudaMemcpy(cur.data(), b.dArgs, sizeof(SweepArgs) * ns, cudaMemcpyDeviceToHost);
    if (r == cudaSuccess && b.chains) {
        curC.resize(ns);
        r = cudaMemcpy(curC.data(), b.dArgsC, sizeof(SweepArgs) * ns, cudaMemcpyDeviceToHost);
    }
    if (r != cudaSuccess) return cudaFail(r, "sweep arguments");
    for (int k = 0; k < ns; ++k) {
        SweepEngine* e = b.sys[k]->engine;
        e->args.temper = cur[k].temper;
        e->args.s.n = cur[k].s.n;
        b.sys[k]->d.n = cur[k].s.n;
        e->runParams.temper = cur[k].temper;
        if (b.chains) {
            e->ch.args.temper = curC[k].temper;
            e->ch.args.s.n = curC[k].s.n;
            e->ch.args.chainFrac = curC[k].chainFrac;
        }
    }
    return SC_OK;
}

// A grand-canonical system whose free slots ran out (its host arguments synchronised):
// larger state arrays and per-particle buffers, the new pointers in its arguments.  The
// caller uploads the batch's arguments afterwards.
static int growSystem(Context* c) {
    SweepEngine* e = c->engine;
    const int newCap = std::max(2 * c->cap, c->cap + 256);
    int rc;
    if ((rc = c->grow(newCap))) return rc;
    if ((rc = particleBuffers(e, newCap))) return rc;
    SweepArgs& a = e->args;
    a.s = c->d;
    a.cellIdx = e->cellIdx; a.cellPosF = e->cellPosF; a.cellDirF = e->cellDirF; a.cellPatF = e->cellPatF;
    a.cellOf = e->cellOf;
    if (e->ch.on) {
        SweepArgs& ac = e->ch.args;
        ac.s = c->d;
        ac.cellIdx = e->ch.cellIdx; ac.cellOf = e->ch.cellOf; ac.slotOf = e->ch.slotOf; ac.cellPosF = e->ch.cellPosF;
    }
    cudaError_t r = cudaMemcpy(&e->gc->cap, &newCap, sizeof newCap, cudaMemcpyHostToDevice);
    if (r != cudaSuccess) return cudaFail(r, "grand-canonical capacity");
    return SC_OK;
}

// Device state, grid and arguments of one system for a run with parameters p.
static int prepareSystem(Context* c, const sc_run_params& p, bool npt) {
    const bool hostChanged = c->hostNewer;    // the running energy must be recomputed
    int rc = c->ensureDevice();
    if (rc) return rc;
    if ((rc = wlPrepare(c, hostChanged))) return rc;
    if (hostChanged && c->engine) c->engine->energyKnown = false;
    SweepEngine* e = c->engine;
    if (!e) {
        e = new SweepEngine();
        c->engine = e;
        if ((rc = engineAlloc(e, (void**)&e->ctl, sizeof(Control)))) return rc;
        if ((rc = particleBuffers(e, std::max(c->cap, 1)))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->counters, sizeof(unsigned long long) * C_COUNT))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->err, sizeof(int)))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->typeCtr, sizeof(unsigned long long) * kTypeCtrCount))) return rc;
        if ((rc = engineAlloc(e, (void**)&e->tinit, sizeof(TypeInit) * MAX_DEV_TYPES))) return rc;
        TypeInit ti[MAX_DEV_TYPES];
        std::memset(ti, 0, sizeof ti);
        for (size_t k = 0; k < c->usedTypes.size() && k < (size_t)MAX_DEV_TYPES; ++k) {
            const IaParam& ia = c->topo.ia[c->usedTypes[k]][c->usedTypes[k]];
            ti[k].geo = ia.geotype[0];
            ti[k].pcos0 = ia.pcoshalfi[0]; ti[k].psin0 = ia.psinhalfi[0];
            ti[k].pcos2 = ia.pcoshalfi[2]; ti[k].psin2 = ia.psinhalfi[2];
            ti[k].csec = ia.csecpatchrot[0]; ti[k].ssec = ia.ssecpatchrot[0];
            ti[k].chcos = ia.chiral_cos[0]; ti[k].chsin = ia.chiral_sin[0];
        }
        cudaMemcpy(e->tinit, ti, sizeof ti, cudaMemcpyHostToDevice);
        Control z;
        std::memset(&z, 0, sizeof z);
        cudaMemcpy(e->ctl, &z, sizeof z, cudaMemcpyHostToDevice);
    }
    if (e->slots < c->cap && (rc = particleBuffers(e, c->cap))) return rc;   // the state grew
    if (e->seed != p.seed) {
        // a new seed restarts the sweep counter of the Philox streams
        unsigned long long zero = 0;
        cudaMemcpy(&e->ctl->sweep, &zero, sizeof zero, cudaMemcpyHostToDevice);
        e->seed = p.seed;
    }
    double box[3];
    cudaMemcpy(box, c->d.box, sizeof box, cudaMemcpyDeviceToHost);
    e->margin = npt ? 0.03 : 1e-9;
    // Wang-Landau: the order parameters' particles diffuse as fast as the cells let them
    // (a displacement that leaves its cell is rejected), so an automatic reach is 1, the
    // widest cells
    e->stencil = chooseStencil(box, c->topo.maxcut, p.stencil == 0 && wlActive(c) ? 1 : p.stencil);
    if ((rc = ensureGrid(c, e, box))) return rc;
    if ((rc = prepareGrand(c, e, p))) return rc;
    e->runParams = p;
    fillArgs(c, e, p);
    if ((rc = prepareChains(c, e, p, box))) return rc;
    cudaMemset(e->counters, 0, sizeof(unsigned long long) * C_COUNT);
    cudaMemset(e->typeCtr, 0, sizeof(unsigned long long) * kTypeCtrCount);
    cudaMemset(e->err, 0, sizeof(int));
    cudaMemset(&e->ctl->maxDrift, 0, sizeof(double));
    cudaMemset(&e->ctl->daErr2, 0, 2 * sizeof(double));
    return SC_OK;
}

static int uploadArgs(Batch& b) {
    int ns = (int)b.sys.size();
    if (ns > b.nArgsAlloc) {
        int rc = b.alloc((void**)&b.dArgs, sizeof(SweepArgs) * ns);
        if (rc) return rc;
        b.nArgsAlloc = ns;
    }
    b.hArgs.resize(ns);
    b.maxN = b.maxCells = b.maxActive = b.maxColours = 0;
    for (int k = 0; k < ns; ++k) {
        b.hArgs[k] = b.sys[k]->engine->args;
        // grand-canonical systems: grids over every slot (the count changes on the device)
        b.maxN = std::max(b.maxN, b.hArgs[k].gc ? b.sys[k]->cap : b.hArgs[k].s.n);
        b.maxCells = std::max(b.maxCells, b.hArgs[k].g.ncells);
        b.maxActive = std::max(b.maxActive, b.hArgs[k].g.nactive);
        b.maxColours = std::max(b.maxColours, b.hArgs[k].g.ncolours);
    }
    cudaError_t r = cudaMemcpy(b.dArgs, b.hArgs.data(), sizeof(SweepArgs) * ns, cudaMemcpyHostToDevice);
    if (r != cudaSuccess) return cudaFail(r, "upload sweep arguments");
    b.wl = false;
    b.switching = false;
    for (const SweepArgs& h : b.hArgs) {
        b.wl |= (h.wl != nullptr);
        b.switching |= (h.swTab != nullptr);
    }
    int on = 0;
    for (Context* c : b.sys) on += c->engine->ch.on ? 1 : 0;
    if (on != 0 && on != ns) return fail(SC_ERR_UNSUPPORTED, "chain moves need every system of a batch to hold chains");
    b.chains = on > 0;
    if (b.chains) {
        if (ns > b.nArgsCAlloc) {
            int rc = b.alloc((void**)&b.dArgsC, sizeof(SweepArgs) * ns);
            if (rc) return rc;
            b.nArgsCAlloc = ns;
        }
        b.hArgsC.resize(ns);
        b.maxCellsC = b.maxActiveC = b.maxColoursC = 0;
        for (int k = 0; k < ns; ++k) {
            SweepEngine* e = b.sys[k]->engine;
            e->ch.args.temper = b.hArgs[k].temper;      // the replica's current temperature
            b.hArgsC[k] = e->ch.args;
            b.maxCellsC = std::max(b.maxCellsC, e->ch.g.ncells);
            b.maxActiveC = std::max(b.maxActiveC, e->ch.g.nactive);
            b.maxColoursC = std::max(b.maxColoursC, e->ch.g.ncolours);
        }
        r = cudaMemcpy(b.dArgsC, b.hArgsC.data(), sizeof(SweepArgs) * ns, cudaMemcpyHostToDevice);
        if (r != cudaSuccess) return cudaFail(r, "upload chain arguments");
    }
    return SC_OK;
}

// Counters / statistics of one system after a run.
static void collectStats(Context* c, sc_run_stats& st) {
    SweepEngine* e = c->engine;
    unsigned long long ctr[C_COUNT];
    Control hc;
    cudaMemcpy(ctr, e->counters, sizeof ctr, cudaMemcpyDeviceToHost);
    // the run's acceptance per type into the Disp records (Updater::optimizeStep reads them)
    unsigned long long tc[kTypeCtrCount];
    cudaMemcpy(tc, e->typeCtr, sizeof tc, cudaMemcpyDeviceToHost);
    for (int t = 0; t < MAXT; ++t) c->trans[t].acc = c->trans[t].rej = c->rot[t].acc = c->rot[t].rej = 0;
    for (size_t k = 0; k < c->usedTypes.size() && k < (size_t)MAX_DEV_TYPES; ++k) {
        const int t = c->usedTypes[k];
        c->trans[t].acc = (long)tc[4 * k]; c->trans[t].rej = (long)tc[4 * k + 1];
        c->rot[t].acc = (long)tc[4 * k + 2]; c->rot[t].rej = (long)tc[4 * k + 3];
    }
    for (int m = 0; m < kMaxChainTypes; ++m) {
        c->chainm[m].acc = (long)tc[kTypeCtrChain + 4 * m]; c->chainm[m].rej = (long)tc[kTypeCtrChain + 4 * m + 1];
        c->chainr[m].acc = (long)tc[kTypeCtrChain + 4 * m + 2]; c->chainr[m].rej = (long)tc[kTypeCtrChain + 4 * m + 3];
    }
    c->edge.acc = (long)ctr[C_ACC_V];
    c->edge.rej = (long)ctr[C_REJ_V];
    cudaMemcpy(&hc, e->ctl, sizeof hc, cudaMemcpyDeviceToHost);
    st.moves = (long)ctr[C_MOVES];
    st.acc_trans = (long)ctr[C_ACC_T]; st.rej_trans = (long)ctr[C_REJ_T];
    st.acc_rot = (long)ctr[C_ACC_R]; st.rej_rot = (long)ctr[C_REJ_R];
    st.acc_vol = (long)ctr[C_ACC_V]; st.rej_vol = (long)ctr[C_REJ_V]; st.vol_constrained = (long)ctr[C_VOL_CONSTR];
    st.pairs_tested = (long)ctr[C_TESTED];
    st.pairs_evaluated = (long)ctr[C_EVAL];
    st.acc_chain = (long)ctr[C_ACC_CH];
    st.rej_chain = (long)ctr[C_REJ_CH];
    st.da_stage1_rejected = (long)ctr[C_S1_REJ];
    st.da_stage2_tried = (long)ctr[C_S2_TRIED];
    st.da_stage2_rejected = (long)ctr[C_S2_REJ];
    st.acc_switch = (long)ctr[C_ACC_SW];
    st.rej_switch = (long)ctr[C_REJ_SW];
    st.da_err_rms = ctr[C_S2_TRIED] ? std::sqrt(hc.daErr2 / (double)ctr[C_S2_TRIED]) : 0.0;
    st.da_err_mean = ctr[C_S2_TRIED] ? hc.daErrSum / (double)ctr[C_S2_TRIED] : 0.0;
    st.energy = hc.energy;
    st.energy_check = hc.energyCheck;
    st.max_drift = hc.maxDrift;
}

static int systemErrors(Context* c) {
    int err = 0;
    cudaMemcpy(&err, c->engine->err, sizeof err, cudaMemcpyDeviceToHost);
    if (err & E_PARTNER_FAR) return fail(SC_ERR_DEVICE, "a bonded partner lies beyond the cell stencil (bond longer than maxcut)");
    if (err & E_FLOW_WAIT) return fail(SC_ERR_DEVICE, "dataflow sweep: a cell waited too long for its neighbours");
    if (err & E_GC_FULL) return fail(SC_ERR_DEVICE, "grand-canonical insertion found no free particle slot");
    return SC_OK;
}

struct RunOut {
    double seconds = 0, phaseSeconds = 0;
    long launches = 0, phaseLaunches = 0;
    long sweeps = 0;        // sweeps run (fewer than asked when Wang-Landau converged)
};

// Runs nsweeps sweeps of every system of the batch; with exchangeEvery > 0 a replica
// exchange follows every exchangeEvery sweeps.
static int runBatch(Batch& b, const sc_run_params& p, long nsweeps, int exchangeEvery, uint64_t exSeed, RunOut& out) {
    const int ns = (int)b.sys.size();
    const bool npt = p.volume_every > 0;
    cudaStream_t s = b.stream;
    cudaError_t r;
    int rc;
    long launches = 0;
    double phaseMs = 0;
    long phaseLaunches = 0;
    if (!b.ev0) {
        cudaEventCreate(&b.ev0); cudaEventCreate(&b.ev1);
    }
    // time_phases: one pair of events per sweep, read after the run (no synchronisation
    // inside the sweeps, so the timed launches run as they would untimed)
    int phaseEvents = 0;
    if (p.time_phases) {
        const size_t want = 2 * (size_t)std::min<long>(nsweeps, 4096);
        while (b.evPhase.size() < want) {
            cudaEvent_t e;
            if ((r = cudaEventCreate(&e)) != cudaSuccess) return cudaFail(r, "phase events");
            b.evPhase.push_back(e);
        }
    }
    // the kernels' shared-memory limits are set once per device (an attribute of the
    // device's context)
    static unsigned long long attrSet = 0;
    const unsigned long long devBit = 1ull << (b.device & 63);
    if (!(attrSet & devBit)) {
        if ((r = cudaFuncSetAttribute(kColour, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDynSmemSurrogate)) !=
            cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kColourDense, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kDynSmemSurrogate)) != cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kColourFlow, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kDynSmemSurrogate)) != cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kColourFlowDense, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kDynSmemSurrogate)) != cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kCellEnergy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDynSmemCell)) !=
            cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kChainColour, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDynSmem)) !=
            cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kChainFlow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDynSmem)) !=
            cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kWlCells, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDynSmemColour)) !=
            cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kCellWarpsFlow, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kDynSmemWarps)) != cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        if ((r = cudaFuncSetAttribute(kCellWarpsFlowDense, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kDynSmemWarps)) != cudaSuccess)
            return cudaFail(r, "shared memory attribute");
        attrSet |= devBit;
    }
    // resident CTAs per SM of the warp-per-cell kernels (their grids are persistent)
    static int warpBlocks[2][64] = {};
    if (!warpBlocks[0][b.device & 63]) {
        int nb0 = 0, nb1 = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb0, kCellWarpsFlow, kCellWarps * 32, kDynSmemWarps);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb1, kCellWarpsFlowDense, kCellWarps * 32, kDynSmemWarps);
        warpBlocks[0][b.device & 63] = std::max(1, nb0);
        warpBlocks[1][b.device & 63] = std::max(1, nb1);
    }
    auto dims = [&](int x) { return dim3((unsigned)std::max(1, x), (unsigned)ns); };
    // systems with a surrogate stage their candidates' FP32 axes and patches as well
    bool anySurrogate = false;
    for (const SweepArgs& h : b.hArgs) anySurrogate |= (h.mlp != nullptr);
    const size_t colourSmem = anySurrogate ? kDynSmemSurrogate : kDynSmemColour;
    const bool dense = (p.variant & 1) != 0;
    // dataflow sweep: one launch per sweep, CTAs per system so that the batch fills the SMs
    // (two CTAs per SM at up to 255 registers, three at 170)
    const bool warpCells = (p.variant & 8) != 0;          // one warp per cell (a dataflow sweep)
    const bool flow = (p.variant & 4) != 0 || warpCells;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b.sys[0]->device);
    const int flowCtas = std::max(1, std::min(b.maxColours * b.maxActive, std::max(1, sms) * (dense ? 3 : 2) / ns));
    const int warpCtas = std::max(1, std::min((b.maxColours * b.maxActive + kCellWarps - 1) / kCellWarps,
                                              std::max(1, sms) * warpBlocks[dense ? 1 : 0][b.device & 63] / ns));
    auto launchCellsOf = [&](const SweepArgs* args, int maxCells) -> cudaError_t {
        kZeroCounts<<<dims((maxCells + 255) / 256), 256, 0, s>>>(args);
        kAssign<<<dims((b.maxN + 255) / 256), 256, 0, s>>>(args);
        kScan<<<dims(1), kScanThreads, 0, s>>>(args);
        kScatter<<<dims((b.maxN + 255) / 256), 256, 0, s>>>(args);
        kSortCells<<<dims((maxCells + 127) / 128), 128, 0, s>>>(args);
        launches += 5;
        return cudaGetLastError();
    };
    auto launchCells = [&]() -> cudaError_t { return launchCellsOf(b.dArgs, b.maxCells); };
    auto exactEnergy = [&](bool check) -> cudaError_t {
        kCellEnergy<<<dims(b.maxCells), kCellThreads, kDynSmemCell, s>>>(b.dArgs, 0);
        if (check) kCheckEnergy<<<dims(1), 1024, 0, s>>>(b.dArgs);
        else kSetEnergy<<<dims(1), 1024, 0, s>>>(b.dArgs);
        launches += 2;
        return cudaGetLastError();
    };
    // exact starting energy (Updater::simulate calls initEM + allToAll, updater.cpp:128-131)
    bool need = false;
    for (Context* c : b.sys) need |= (!c->engine->energyKnown || c->hostNewer);
    if (need) {
        kBeginSweep<<<dims(1), 32, 0, s>>>(b.dArgs, 0);
        if ((r = launchCells()) != cudaSuccess) return cudaFail(r, "cell list");
        if ((r = exactEnergy(false)) != cudaSuccess) return cudaFail(r, "energy");
        launches += 1;
        for (Context* c : b.sys) c->engine->energyKnown = true;
    }
    auto launchOne = [&](bool volDue, bool timing) -> cudaError_t {
        kBeginSweep<<<dims(1), 32, 0, s>>>(b.dArgs, volDue ? 1 : 0);
        cudaError_t r2 = launchCells();
        if (r2 != cudaSuccess) return r2;
        const bool timed = timing && 2 * phaseEvents + 1 < (int)b.evPhase.size();
        if (timed) cudaEventRecord(b.evPhase[2 * phaseEvents], s);
        if (warpCells) {
            if (dense) kCellWarpsFlowDense<<<dims(warpCtas), kCellWarps * 32, kDynSmemWarps, s>>>(b.dArgs);
            else kCellWarpsFlow<<<dims(warpCtas), kCellWarps * 32, kDynSmemWarps, s>>>(b.dArgs);
        } else if (flow) {
            if (dense) kColourFlowDense<<<dims(flowCtas), kMoveThreads, colourSmem, s>>>(b.dArgs);
            else kColourFlow<<<dims(flowCtas), kMoveThreads, colourSmem, s>>>(b.dArgs);
        } else {
            for (int ph = 0; ph < b.maxColours; ++ph) {
                if (dense) kColourDense<<<dims(b.maxActive), kMoveThreads, colourSmem, s>>>(b.dArgs, ph);
                else kColour<<<dims(b.maxActive), kMoveThreads, colourSmem, s>>>(b.dArgs, ph);
            }
        }
        if (timed) {
            cudaEventRecord(b.evPhase[2 * phaseEvents + 1], s);
            ++phaseEvents;
        }
        if (timed || !timing) phaseLaunches += flow ? 1 : b.maxColours;
        if (b.switching) {      // type switch moves: a checkerboard phase over the same cells
            for (int ph = 0; ph < b.maxColours; ++ph)
                kSwitchColour<<<dims(b.maxActive), kSwThreads, 0, s>>>(b.dArgs, ph);
            launches += b.maxColours;
        }
        if (b.wl) {         // Wang-Landau: the cells of the order parameters' particles, last
            kWlCells<<<dims(1), kMoveThreads, kDynSmemColour, s>>>(b.dArgs);
            launches += 1;
        }
        kEndSweep<<<dims(1), kEndThreads, 0, s>>>(b.dArgs);
        launches += 2 + (flow ? 1 : b.maxColours);
        if (b.chains) {       // chain moves: their own grid, colours and cell list
            kBeginSweep<<<dims(1), 32, 0, s>>>(b.dArgsC, 0);
            if ((r2 = launchCellsOf(b.dArgsC, b.maxCellsC)) != cudaSuccess) return r2;
            kChainBin<<<dims(1), 1024, 0, s>>>(b.dArgsC);
            if (flow) {
                const int ctas = std::max(1, std::min(b.maxColoursC * b.maxActiveC, std::max(1, sms) * 2 / ns));
                kChainFlow<<<dims(ctas), kMoveThreads, kDynSmem, s>>>(b.dArgsC);
            } else {
                for (int ph = 0; ph < b.maxColoursC; ++ph)
                    kChainColour<<<dims(b.maxActiveC), kMoveThreads, kDynSmem, s>>>(b.dArgsC, ph);
            }
            kEndSweep<<<dims(1), kEndThreads, 0, s>>>(b.dArgsC);
            launches += 3 + (flow ? 1 : b.maxColoursC);
            if (b.wl) {
                kWlAfterChains<<<dims(1), 32, 0, s>>>(b.dArgs);
                launches += 1;
            }
        }
        if (volDue) {
            // chain moves left particles outside the cells of this sweep's list: list them anew
            if (b.chains && (r2 = launchCells()) != cudaSuccess) return r2;
            kCellEnergy<<<dims(b.maxCells), kCellThreads, kDynSmemCell, s>>>(b.dArgs, 1);
            kVolumeAccept<<<dims(1), 256, 0, s>>>(b.dArgs);
            launches += 2;
        }
        if (b.wl) {
            kWlEndSweep<<<dims(1), 256, 0, s>>>(b.dArgs);
            launches += 1;
        }
        return cudaGetLastError();
    };
    cudaEventRecord(b.ev0, s);
    // Blocks of G sweeps are captured once into a CUDA graph and replayed: the kernels
    // read what changes between sweeps (sweep index, grid offset, colour order, box,
    // energy, temperature) from device memory.
    const int ve = npt ? p.volume_every : 1;
    long G = (long)ve * std::max(1, (8 + ve - 1) / ve);
    if (exchangeEvery > 0) G = std::max(1L, std::min(G, (long)exchangeEvery));
    // grand-canonical moves: after every grand_every-th sweep of the call (updater.cpp:164-165),
    // between the captured blocks; the host keeps a free slot for every insertion
    std::vector<long> nUpper(ns, -1);      // bound on each grand-canonical system's device count
    bool gc = false;
    if (p.grand_every > 0)
        for (int k = 0; k < ns; ++k)
            if (b.hArgs[k].gc) { gc = true; nUpper[k] = b.hArgs[k].s.n; }
    long nextGc = gc ? p.grand_every - (long)(p.sweep_offset % p.grand_every) : -1;
    if (gc) G = std::max(1L, std::min(G, (long)p.grand_every));
    const bool useGraph = !p.time_phases;
    const long chunk = 48;
    long nextCheck = p.check_every > 0 ? p.check_every : -1;
    long nextRegrid = npt ? chunk : -1;
    long nextExchange = exchangeEvery > 0 ? exchangeEvery : -1;
    // Wang-Landau: the flatness check runs every kWlUpdateEvery sweeps of the device's count;
    // the host looks for convergence at those sweeps and stops there, as the reference does
    long nextWl = -1;
    if (b.wl) {
        unsigned long long done = 0;
        cudaMemcpy(&done, &b.sys[0]->engine->ctl->sweep, sizeof done, cudaMemcpyDeviceToHost);
        nextWl = (long)(kWlUpdateEvery - (long)(done % kWlUpdateEvery));
        bool allDone = true;
        for (Context* c : b.sys) allDone &= wlConverged(c);
        if (allDone) {              // an earlier call's flatness check ended the run
            out.sweeps = 0;
            return SC_OK;
        }
    }
    out.sweeps = nsweeps;
    long sw = 0;
    while (sw < nsweeps) {
        long left = nsweeps - sw;
        bool aligned = (sw % G == 0) && (nextExchange < 0 || nextExchange - sw >= G) && (nextWl < 0 || nextWl - sw >= G) &&
                       (nextGc < 0 || nextGc - sw >= G);
        if (useGraph && left >= G && aligned) {
            int key[16] = {ns, b.maxN, b.maxCells, b.maxActive, b.maxColours, (int)G, anySurrogate ? 1 : 0,
                           b.chains ? 1 : 0, b.maxCellsC, b.maxActiveC, b.maxColoursC, dense ? 1 : 0, flow ? 1 : 0,
                           b.wl ? 1 : 0, warpCells ? 1 : 0, b.switching ? 1 : 0};
            if (!b.graph || std::memcmp(key, b.graphDims, sizeof key) != 0) {
                if (b.graph) { cudaGraphExecDestroy(b.graph); b.graph = nullptr; }
                cudaGraph_t graph;
                long before = launches, beforeP = phaseLaunches;
                if ((r = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cudaFail(r, "graph capture");
                for (long k = 0; k < G; ++k) {
                    cudaError_t r2 = launchOne(npt && ((k + 1) % ve == 0), false);
                    if (r2 != cudaSuccess) { cudaStreamEndCapture(s, &graph); return cudaFail(r2, "graph capture launch"); }
                }
                if ((r = cudaStreamEndCapture(s, &graph)) != cudaSuccess) return cudaFail(r, "graph capture end");
                r = cudaGraphInstantiate(&b.graph, graph, 0);
                cudaGraphDestroy(graph);
                if (r != cudaSuccess) return cudaFail(r, "graph instantiate");
                b.graphLaunches = launches - before;
                b.graphPhaseLaunches = phaseLaunches - beforeP;
                launches = before;
                phaseLaunches = beforeP;
                std::memcpy(b.graphDims, key, sizeof key);
            }
            if ((r = cudaGraphLaunch(b.graph, s)) != cudaSuccess) return cudaFail(r, "graph launch");
            launches += b.graphLaunches;
            phaseLaunches += b.graphPhaseLaunches;
            sw += G;
        } else {
            if ((r = launchOne(npt && ((sw + 1) % ve == 0), p.time_phases != 0)) != cudaSuccess) return cudaFail(r, "sweep launch");
            sw += 1;
        }
        if (nextWl > 0 && sw >= nextWl) {
            while (nextWl <= sw) nextWl += kWlUpdateEvery;
            if ((r = cudaStreamSynchronize(s)) != cudaSuccess) return cudaFail(r, "sweep");
            bool allDone = true;
            for (Context* c : b.sys) allDone &= wlConverged(c);
            if (allDone) { out.sweeps = sw; break; }
        }
        if (nextExchange > 0 && sw >= nextExchange) {
            kExchange<<<1, 32, 0, s>>>(b.dArgs, b.chains ? b.dArgsC : nullptr, b.dLadder, b.dLadderStart, b.nLadders,
                                       exSeed, b.dExCtr);
            launches += 1;
            while (nextExchange <= sw) nextExchange += exchangeEvery;
        }
        if (nextGc > 0 && sw >= nextGc) {
            while (nextGc <= sw) nextGc += p.grand_every;
            bool full = false;
            for (int k = 0; k < ns; ++k) full |= nUpper[k] >= 0 && nUpper[k] + 1 > b.sys[k]->cap;
            if (full) {          // read the counts; grow the systems that have no free slot
                if ((r = cudaStreamSynchronize(s)) != cudaSuccess) return cudaFail(r, "sweep");
                if ((rc = syncDeviceArgs(b))) return rc;
                bool grown = false;
                for (int k = 0; k < ns; ++k) {
                    if (nUpper[k] < 0) continue;
                    nUpper[k] = b.sys[k]->d.n;
                    if (nUpper[k] + 1 > b.sys[k]->cap) {
                        if ((rc = growSystem(b.sys[k]))) return rc;
                        grown = true;
                    }
                }
                if (grown && (rc = uploadArgs(b))) return rc;
            }
            kGrandCanon<<<dims(1), kGcThreads, 0, s>>>(b.dArgs, b.chains ? b.dArgsC : nullptr);
            launches += 1;
            for (int k = 0; k < ns; ++k)
                if (nUpper[k] >= 0) nUpper[k] += 1;
        }
        if (nextCheck > 0 && sw >= nextCheck) {
            // the cell list (box fractions) stays valid after an accepted volume move, not after
            // chain moves (particles left their cells) or grand-canonical moves (slots moved):
            // then it is built anew, on the sweep's grid
            if ((b.chains || gc) && (r = launchCells()) != cudaSuccess) return cudaFail(r, "cell list");
            if ((r = exactEnergy(true)) != cudaSuccess) return cudaFail(r, "energy check");
            while (nextCheck <= sw) nextCheck += p.check_every;
        }
        if (nextRegrid > 0 && sw >= nextRegrid && sw < nsweeps) {
            // the box changed on the device: re-derive the cell grids when needed
            while (nextRegrid <= sw) nextRegrid += chunk;
            if ((r = cudaStreamSynchronize(s)) != cudaSuccess) return cudaFail(r, "sweep");
            // an upload below must keep the device's temperatures and counts, for every system
            if ((rc = syncDeviceArgs(b))) return rc;
            bool changed = false;
            for (int k = 0; k < ns; ++k) {
                Context* c = b.sys[k];
                SweepEngine* e = c->engine;
                double box[3];
                cudaMemcpy(box, c->d.box, sizeof box, cudaMemcpyDeviceToHost);
                Grid ng = makeGrid(box, c->topo.maxcut, e->margin, e->stencil);
                const bool mainChanged = ng.nc[0] != e->g.nc[0] || ng.nc[1] != e->g.nc[1] || ng.nc[2] != e->g.nc[2];
                if (mainChanged || e->ch.on) {
                    if (mainChanged && (rc = ensureGrid(c, e, box))) return rc;
                    // the system's own parameters, at the temperature it has now
                    sc_run_params q = e->runParams;
                    Grid oldC = e->ch.g;
                    fillArgs(c, e, q);
                    if (e->ch.on) {
                        if ((rc = prepareChains(c, e, q, box))) return rc;
                        changed |= e->ch.g.nc[0] != oldC.nc[0] || e->ch.g.nc[1] != oldC.nc[1] ||
                                   e->ch.g.nc[2] != oldC.nc[2];
                    }
                    changed |= mainChanged;
                }
            }
            if (changed && (rc = uploadArgs(b))) return rc;
        }
        if ((r = cudaGetLastError()) != cudaSuccess) return cudaFail(r, "sweep launch");
    }
    cudaEventRecord(b.ev1, s);
    if ((r = cudaStreamSynchronize(s)) != cudaSuccess) return cudaFail(r, "sweep");
    float ms = 0;
    cudaEventElapsedTime(&ms, b.ev0, b.ev1);
    out.seconds = ms * 1e-3;
    for (int k = 0; k < phaseEvents; ++k) {
        float pms = 0;
        cudaEventElapsedTime(&pms, b.evPhase[2 * k], b.evPhase[2 * k + 1]);
        phaseMs += pms;
    }
    out.phaseSeconds = phaseMs * 1e-3;
    out.launches = launches;
    out.phaseLaunches = phaseLaunches;
    for (Context* c : b.sys) c->devNewer = true;
    return SC_OK;
}

// Moves of the options that the GPU loop does not make.
static int checkMoves(const Context* c) {
    (void)c;
    return SC_OK;
}

static int checkParams(const sc_run_params& p) {
    if (p.nsweeps < 0) return fail(SC_ERR_ARG, "nsweeps must be >= 0");
    if (!(p.temper > 0)) return fail(SC_ERR_ARG, "temper must be positive");
    if (p.ptype < 0 || p.ptype > 5) return fail(SC_ERR_ARG, "ptype must be 0..5 (movecreator.cpp:349-546)");
    if (p.stencil < 0 || p.stencil > 3) return fail(SC_ERR_ARG, "stencil must be 0 (auto), 1, 2 or 3");
    if (p.variant < -1 || p.variant > 15) return fail(SC_ERR_ARG, "variant must be -1 (tuned) or 0..15");
    if (p.variant > 0 && (p.variant & 8) && p.delayed)
        return fail(SC_ERR_UNSUPPORTED, "the warp-per-cell kernel (variant bit 3) runs plain moves only");
    if (p.flow_wait_polls < 0) return fail(SC_ERR_ARG, "flow_wait_polls must be >= 0");
    if (p.grand_every < 0) return fail(SC_ERR_ARG, "grand_every must be >= 0");
    if (p.sweep_offset < 0) return fail(SC_ERR_ARG, "sweep_offset must be >= 0");
    if (!(p.switchprob >= 0.0)) return fail(SC_ERR_ARG, "switchprob must be >= 0");
    return SC_OK;
}

// variant = -1: the reach and kernel variant sc_tune measured fastest for this context and
// mode (stencil 0 takes the tuned reach; an explicit stencil is kept), else the dataflow
// sweep with the default reach.
static sc_run_params resolveTuned(const Context* c, const sc_run_params& p) {
    sc_run_params q = p;
    if (p.variant != -1) return q;
    const int m = p.delayed ? 1 : 0;
    q.variant = c->tunedVariant[m] >= 0 ? c->tunedVariant[m] : 4;
    if (p.stencil == 0 && c->tunedVariant[m] >= 0) q.stencil = c->tunedStencil[m];
    return q;
}

int runSweeps(Context* c, const sc_run_params& p0, sc_run_stats& st) {
    std::memset(&st, 0, sizeof st);
    int rc = checkParams(p0);
    if (rc) return rc;
    const sc_run_params p = resolveTuned(c, p0);
    const bool grandRun = p.grand_every > 0 && !c->grand.empty();
    if (c->conf.p.empty() && !grandRun) return SC_OK;     // an empty grand-canonical box can fill up
    if (grandRun && wlActive(c))
        return fail(SC_ERR_UNSUPPORTED, "grand-canonical moves with Wang-Landau weights are outside the GPU path");
    if (p.switchprob > 0.0 && c->anySwitch && wlActive(c))
        return fail(SC_ERR_UNSUPPORTED, "type switch moves with Wang-Landau weights (WangLandau::runSwitch) are outside the "
                                        "GPU path");
    if (p.delayed && !c->surrogate) return fail(SC_ERR_STATE, "delayed = 1 needs a surrogate (sc_set_surrogate)");
    if ((rc = checkMoves(c))) return rc;
    if ((rc = wlCheckRun(c, p))) return rc;
    if ((p.variant & 8) && wlActive(c))
        return fail(SC_ERR_UNSUPPORTED, "the warp-per-cell kernel (variant bit 3) does not run Wang-Landau moves");
    const bool npt = p.volume_every > 0;
    if ((rc = prepareSystem(c, p, npt))) return rc;
    if (!c->batch) {
        c->batch = new Batch();
        c->batch->sys = {c};
        c->batch->stream = c->stream;
        c->batch->device = c->device;
    }
    Batch& b = *c->batch;
    if ((rc = uploadArgs(b))) return rc;
    RunOut out;
    rc = runBatch(b, p, p.nsweeps, 0, 0, out);
    // the device's particle vector, whatever happened (a failed run leaves it consistent too)
    const int rcG = finishGrand(c, b.dArgs);
    if (rc) return rc;
    if (rcG) return rcG;
    collectStats(c, st);
    if (c->engine->gcOn) {
        GcDev h;
        cudaMemcpy(&h, c->engine->gc, sizeof h, cudaMemcpyDeviceToHost);
        for (int k = 0; k < h.nSpecies; ++k) {
            st.acc_insert += (long)h.ctr[k][1]; st.rej_insert += (long)h.ctr[k][2];
            st.acc_delete += (long)h.ctr[k][3]; st.rej_delete += (long)h.ctr[k][4];
        }
    }
    st.particles = (long)c->conf.p.size();
    st.sweeps = out.sweeps;
    st.seconds = out.seconds;
    st.phase_seconds = out.phaseSeconds;
    st.phase_launches = out.phaseLaunches;
    st.launches = out.launches;
    c->lastLaunches = out.launches;
    rc = systemErrors(c);
    // a sweep that stopped early (a dataflow wait gave up, a partner lay beyond the stencil) leaves cells
    // unmoved and their energy changes unsummed: the next run recomputes the exact energy
    if (rc) c->engine->energyKnown = false;
    return rc;
}

// The candidate screens of the move kernels over every (target, particle) pair: the pairs
// that pass stage A, with stage B's verdict (kScreenSurvivors).
int screenSurvivors(Context* c, int ntargets, const int* targets, long cap, int* I, int* J, unsigned char* B,
                    long* count) {
    int rc = c->ensureDevice();
    if (rc) return rc;
    const int n = (int)c->conf.p.size();
    if (ntargets < 0 || (!targets && ntargets != n)) return fail(SC_ERR_ARG, "sc_screen_survivors: targets");
    for (int k = 0; targets && k < ntargets; ++k)
        if (targets[k] < 0 || targets[k] >= n) return fail(SC_ERR_ARG, "sc_screen_survivors: target out of range");
    int *dT = nullptr, *dI = nullptr, *dJ = nullptr;
    unsigned char* dB = nullptr;
    unsigned long long* dN = nullptr;
    const long capd = std::max(cap, 1L);
    cudaError_t e = cudaSuccess;
    auto freeAll = [&]() { cudaFree(dT); cudaFree(dI); cudaFree(dJ); cudaFree(dB); cudaFree(dN); };
    if (targets) e = cudaMalloc(&dT, sizeof(int) * std::max(ntargets, 1));
    if (e == cudaSuccess) e = cudaMalloc(&dI, sizeof(int) * capd);
    if (e == cudaSuccess) e = cudaMalloc(&dJ, sizeof(int) * capd);
    if (e == cudaSuccess) e = cudaMalloc(&dB, capd);
    if (e == cudaSuccess) e = cudaMalloc(&dN, sizeof(unsigned long long));
    if (e == cudaSuccess && targets)
        e = cudaMemcpyAsync(dT, targets, sizeof(int) * ntargets, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(dN, 0, sizeof(unsigned long long), c->stream);
    if (e != cudaSuccess) { freeAll(); return cudaFail(e, "sc_screen_survivors: buffers"); }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    kScreenSurvivors<<<std::max(1, sms) * 8, 256, 0, c->stream>>>(c->d, c->tables, dT, ntargets, cap, dI, dJ, dB, dN);
    unsigned long long cnt = 0;
    e = cudaMemcpyAsync(&cnt, dN, sizeof cnt, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    const long got = (long)std::min<unsigned long long>(cnt, (unsigned long long)cap);
    if (e == cudaSuccess && got > 0) {
        e = cudaMemcpy(I, dI, sizeof(int) * got, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(J, dJ, sizeof(int) * got, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(B, dB, got, cudaMemcpyDeviceToHost);
    }
    freeAll();
    if (e != cudaSuccess) return cudaFail(e, "sc_screen_survivors");
    *count = (long)cnt;
    if ((long long)cnt > (long long)cap) return fail(SC_ERR_RANGE, "sc_screen_survivors: more survivors than cap");
    return SC_OK;
}

// ---- step-size adaptation --------------------------------------------------------------
// Updater::optimizeStep (scOOP/mc/updater.cpp:395-429): the change of the maximum step keeps
// its direction while mx * acceptance grows and turns back when it falls; no accepted move
// shrinks the step; bounds [lo, hi]; the counts restart.
static void optimizeStep(Context::Disp& x, double hi, double lo) {
    const double ratio = (x.acc + x.rej) > 0 ? (double)x.acc / (double)(x.acc + x.rej) : 0.0;
    const double now = x.mx * ratio;
    if (x.oldrmsd > 0) {
        const bool worse = now < x.oldrmsd, grew = x.oldmx > 1;
        if (worse == grew) { x.mx /= 1.05; x.oldmx = 0.95; }
        else { x.mx *= 1.05; x.oldmx = 1.05; }
    }
    if (now > 0) {
        x.oldrmsd = now;
    } else {
        x.oldrmsd = 0.0;
        x.mx /= 1.05;
        x.oldmx = 0.95;
    }
    if (x.mx > hi) x.mx = hi;
    if (x.mx < lo) x.mx = lo;
    x.acc = x.rej = 0;
}

// Updater::optimizeRot (updater.cpp:431-464): the same on cos(maximum angle), in 1 % steps
// (mx is a cosine: a larger rotation is a smaller mx).
static void optimizeRot(Context::Disp& x, double hi, double lo) {
    const double ratio = (x.acc + x.rej) > 0 ? (double)x.acc / (double)(x.acc + x.rej) : 0.0;
    const double now = x.mx * ratio;
    if (x.oldrmsd > 0) {
        const bool better = now > x.oldrmsd, grew = x.oldmx > 1;
        if (better == grew) { x.mx *= 0.99; x.oldmx *= 0.99; }
        else { x.mx *= 1.01; x.oldmx *= 1.01; }
    }
    if (now > 0) {
        x.oldrmsd = now;
    } else {
        x.oldrmsd = 0.0;
        x.mx *= 1.01;
        x.oldmx = 1.01;
    }
    if (x.mx > hi) x.mx = hi;
    if (x.mx < lo) x.mx = lo;
    x.acc = x.rej = 0;
}

// The Disp records start from the options (Sim::readOptions, sim.h:359-373): displacement
// per type, cos of the maximum rotation, chain steps, box edge range.
void initStepSizes(Context* c) {
    if (c->stepsInit) return;
    const double pih = 1.57079632679489661923132169163975;
    // (the acceptance counts of a run already made stay: they feed the first adjustment)
    auto start = [](Context::Disp& d, double mx) { d.mx = mx; d.oldrmsd = 0.0; d.oldmx = 0.0; };
    for (int t = 0; t < MAXT; ++t) {
        start(c->trans[t], c->opts.trans_type[t]);
        start(c->rot[t], cos(c->opts.rotmx_deg / 180.0 * pih));
    }
    for (int m = 0; m < Context::kMaxChainSteps; ++m) {
        start(c->chainm[m], c->opts.chainmmx);
        start(c->chainr[m], cos(c->opts.chainrmx_deg / 180.0 * pih));
    }
    start(c->edge, c->opts.edge_mx);
    c->stepsInit = true;
}

// The adjustment block of Updater::simulate (updater.cpp:238-253) on the last run's counts:
// optimizeStep on the displacement of every type and chain molecule type that moved (hi 1.5),
// optimizeRot on their rotation records (5.0, 0.01), optimizeStep on the box edge (1.0).  The
// adapted displacements and edge range take effect in later runs; as in the reference, whose
// rotations read Disp::angle and not the adapted cosine, rotations keep the options' angle.
int adjustSteps(Context* c) {
    initStepSizes(c);
    for (int t = 0; t < MAXT; ++t) {
        if (c->trans[t].acc > 0 || c->trans[t].rej > 0) optimizeStep(c->trans[t], 1.5, 0.0);
        if (c->rot[t].acc > 0 || c->rot[t].rej > 0) optimizeRot(c->rot[t], 5.0, 0.01);
    }
    for (int m = 0; m < Context::kMaxChainSteps; ++m) {
        if (c->chainm[m].acc > 0 || c->chainm[m].rej > 0) optimizeStep(c->chainm[m], 1.5, 0.0);
        if (c->chainr[m].acc > 0 || c->chainr[m].rej > 0) optimizeRot(c->chainr[m], 5.0, 0.01);
    }
    optimizeStep(c->edge, 1.0, 0.0);
    for (int t = 0; t < MAXT; ++t) c->opts.trans_type[t] = c->trans[t].mx;
    for (int m = 0; m < Context::kMaxChainSteps; ++m) c->chainAdapted[m] = c->chainm[m].mx;
    c->opts.edge_mx = c->edge.mx;
    ++c->adjustments;
    return SC_OK;
}

// The equilibration of main.cpp:270-287: nequil/2 sweeps with the step adjustment every
// `adjust` sweeps, then nequil/2 sweeps without.  Displacements follow the adapted per-type
// steps; the box edge range is the adapted one.
int equilibrate(Context* c, const sc_run_params& p, long nequil, long adjust, sc_run_stats& st) {
    std::memset(&st, 0, sizeof st);
    if (nequil < 0 || adjust < 0) return fail(SC_ERR_ARG, "sc_equilibrate: nequil and adjust must be >= 0");
    initStepSizes(c);
    const long half = nequil / 2;
    sc_run_params q = p;
    // the reference's two loops (main.cpp:270-287): sweeps, and the grand-canonical schedule,
    // count from each loop's start
    auto run = [&](long n, long offset) -> int {
        q.nsweeps = n;
        q.sweep_offset = offset;
        q.edge_mx = c->edge.mx;
        sc_run_stats s1;
        int rc = runSweeps(c, q, s1);
        if (rc) return rc;
        st.sweeps += s1.sweeps; st.moves += s1.moves;
        st.acc_trans += s1.acc_trans; st.rej_trans += s1.rej_trans; st.acc_rot += s1.acc_rot; st.rej_rot += s1.rej_rot;
        st.acc_vol += s1.acc_vol; st.rej_vol += s1.rej_vol; st.vol_constrained += s1.vol_constrained;
        st.acc_chain += s1.acc_chain; st.rej_chain += s1.rej_chain;
        st.pairs_tested += s1.pairs_tested; st.pairs_evaluated += s1.pairs_evaluated;
        st.seconds += s1.seconds; st.launches += s1.launches;
        st.energy = s1.energy; st.energy_check = s1.energy_check; st.max_drift = std::max(st.max_drift, s1.max_drift);
        st.acc_switch += s1.acc_switch; st.rej_switch += s1.rej_switch;
        st.acc_insert += s1.acc_insert; st.rej_insert += s1.rej_insert;
        st.acc_delete += s1.acc_delete; st.rej_delete += s1.rej_delete;
        st.particles = s1.particles;
        return SC_OK;
    };
    long done = 0;
    while (done < half) {
        const long blk = adjust > 0 ? std::min(adjust, half - done) : half - done;
        int rc = run(blk, done);
        if (rc) return rc;
        done += blk;
        if (adjust > 0 && blk == adjust) adjustSteps(c);     // at sweep == next_adjust
    }
    if (half > 0) {
        int rc = run(half, 0);
        if (rc) return rc;
    }
    return SC_OK;
}

// The tuner: times every (reach, kernel variant) candidate for p's mode on the context's
// current state (restored before every candidate and at the end, so the state the caller
// sees is unchanged; the running energy is recomputed by the next run), and keeps the
// fastest for later runs with variant = -1.  Candidates: reach 1, 2, 3 (cells maxcut/s
// wide: how many cells move at once and how many candidates each stages) times variants
// {colour-phase launches, dataflow sweep} x {lowest latency, more CTAs per SM}, plus paired
// passes and the warp-per-cell dataflow sweep for plain moves.
int tuneSweeps(Context* c, const sc_run_params& p, int sweeps, sc_run_params& best, double* rates, int* ncand) {
    if (sweeps < 1) return fail(SC_ERR_ARG, "sc_tune: sweeps must be >= 1");
    if (wlActive(c)) return fail(SC_ERR_UNSUPPORTED, "sc_tune with Wang-Landau weights: tuning sweeps would change them");
    int rc = checkParams(p);
    if (rc) return rc;
    if (c->conf.p.empty()) return fail(SC_ERR_STATE, "sc_tune: no particles");
    if ((rc = c->ensureDevice())) return rc;
    if ((rc = c->downloadState())) return rc;
    const std::vector<Particle> snap = c->conf.p;
    const Vec3 snapBox = c->conf.box;
    auto restore = [&]() {
        c->conf.p = snap;
        c->conf.box = snapBox;
        c->hostNewer = true;
        c->devNewer = false;
    };
    std::vector<int> variants = p.delayed ? std::vector<int>{0, 1, 4, 5} : std::vector<int>{0, 1, 2, 3, 4, 5, 8, 9};
    if (wlActive(c)) variants = {0, 1, 4, 5};
    double bestRate = -1.0;
    int k = 0;
    best = p;
    for (int reach = 1; reach <= 3; ++reach)
        for (int v : variants) {
            restore();
            sc_run_params q = p;
            q.stencil = reach;
            q.variant = v;
            q.check_every = 0;
            q.time_phases = 0;
            q.grand_every = 0;                 // the candidates move the same particles
            q.switchprob = 0.0;
            q.nsweeps = 2;                     // grid, graph capture, caches
            sc_run_stats st;
            double rate = 0.0;
            if (runSweeps(c, q, st) == SC_OK) {
                q.nsweeps = sweeps;
                if (runSweeps(c, q, st) == SC_OK && st.seconds > 0) rate = (double)st.moves / st.seconds;
            }
            if (rates) rates[k] = rate;
            ++k;
            if (rate > bestRate) {
                bestRate = rate;
                best.stencil = reach;
                best.variant = v;
            }
        }
    restore();
    if (ncand) *ncand = k;
    if (bestRate <= 0.0) return fail(SC_ERR_STATE, "sc_tune: no candidate ran");
    const int m = p.delayed ? 1 : 0;
    c->tunedStencil[m] = best.stencil;
    c->tunedVariant[m] = best.variant;
    return SC_OK;
}

// --- parallel-tempering replicas -----------------------------------------------------

struct ReplicaSet {
    Batch b;
    std::vector<double> temps;      // temperature of each replica at creation
    std::vector<int> group;         // ladder of each replica
    std::vector<int> ladderHost;    // replica at each ladder slot (creation order)
    std::vector<int> ladderStartHost;
};

int createReplicas(Context* const* sys, int nrep, const double* temps, const int* group, void** out) {
    if (nrep < 1) return fail(SC_ERR_ARG, "need at least one replica");
    ReplicaSet* R = new ReplicaSet();
    int device = sys[0]->device;
    for (int k = 0; k < nrep; ++k) {
        if (!sys[k] || !(temps[k] > 0)) { delete R; return fail(SC_ERR_ARG, "null replica or non-positive temperature"); }
        if (sys[k]->device != device) { delete R; return fail(SC_ERR_ARG, "all replicas must use the same device"); }
        for (int q = 0; q < k; ++q)
            if (sys[q] == sys[k]) { delete R; return fail(SC_ERR_ARG, "a context appears twice in the replica set"); }
        R->b.sys.push_back(sys[k]);
        R->temps.push_back(temps[k]);
        R->group.push_back(group ? group[k] : 0);
    }
    // ladders: replicas of one group, ordered by temperature; members must hold the same system
    int ng = 0;
    for (int g : R->group) ng = std::max(ng, g + 1);
    R->ladderStartHost.push_back(0);
    for (int g = 0; g < ng; ++g) {
        std::vector<int> mem;
        for (int k = 0; k < nrep; ++k) if (R->group[k] == g) mem.push_back(k);
        std::sort(mem.begin(), mem.end(), [&](int x, int y) { return R->temps[x] < R->temps[y]; });
        for (size_t q = 1; q < mem.size(); ++q) {
            Context* a = sys[mem[0]];
            Context* c2 = sys[mem[q]];
            if (a->conf.p.size() != c2->conf.p.size() || a->usedTypes != c2->usedTypes) {
                delete R;
                return fail(SC_ERR_ARG, "replicas of one ladder must hold the same system (N and types)");
            }
        }
        for (int k : mem) R->ladderHost.push_back(k);
        R->ladderStartHost.push_back((int)R->ladderHost.size());
    }
    if ((int)R->ladderHost.size() != nrep) { delete R; return fail(SC_ERR_ARG, "ladder ids must be 0..n-1"); }
    *out = R;
    return SC_OK;
}

void destroyReplicas(void* h) { delete static_cast<ReplicaSet*>(h); }

int runReplicas(void* h, const sc_run_params& p0, int exchangeEvery, sc_run_stats& st, double* tempsOut,
                double* energiesOut, long* exTried, long* exAcc) {
    ReplicaSet* R = static_cast<ReplicaSet*>(h);
    std::memset(&st, 0, sizeof st);
    int rc = checkParams(p0);
    if (rc) return rc;
    // a batch has no tuned choice of its own: variant -1 is the dataflow sweep
    sc_run_params p = p0;
    if (p.variant < 0) p.variant = 4;
    Batch& b = R->b;
    const int nrep = (int)b.sys.size();
    const bool npt = p.volume_every > 0;
    DeviceScope dev(b.sys[0]->device);
    for (int k = 0; k < nrep; ++k) {
        Context* c = b.sys[k];
        if (c->conf.p.empty()) return fail(SC_ERR_ARG, "a replica holds no particles");
        if ((rc = checkMoves(c))) return rc;
        if (wlActive(c) && exchangeEvery > 0)
            return fail(SC_ERR_UNSUPPORTED, "Wang-Landau weights with replica exchange (the exchange would need their "
                                            "terms, movecreator.cpp:736-740); walkers run with exchange_every = 0");
        sc_run_params q = p;
        sc_default_run(reinterpret_cast<const sc_context*>(c), &q);   // per-replica step sizes
        q.nsweeps = p.nsweeps; q.seed = p.seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(k + 1);
        q.temper = R->temps[k]; q.ptype = p.ptype; q.volume_every = p.volume_every; q.check_every = p.check_every;
        q.stencil = p.stencil; q.time_phases = p.time_phases; q.press = p.press; q.delayed = p.delayed;
        q.variant = p.variant;
        q.grand_every = c->grand.empty() ? 0 : p.grand_every;
        q.sweep_offset = p.sweep_offset;
        if (q.grand_every > 0) {          // the exchange reads the species of one replica for both
            const Context* c0 = b.sys[0];
            bool same = c0->grand.size() == c->grand.size();
            for (size_t g = 0; same && g < c->grand.size(); ++g)
                same = c0->grand[g].molType == c->grand[g].molType && c0->grand[g].chemPot == c->grand[g].chemPot;
            if (!same) return fail(SC_ERR_UNSUPPORTED, "grand-canonical replicas need the same species and activities");
            if (wlActive(c))
                return fail(SC_ERR_UNSUPPORTED, "grand-canonical moves with Wang-Landau weights are outside the GPU path");
        }
        q.switchprob = c->anySwitch ? p.switchprob : 0.0;
        if (p.delayed && !c->surrogate) return fail(SC_ERR_STATE, "delayed = 1 needs a surrogate on every replica");
        if ((rc = wlCheckRun(c, q))) return rc;
        if ((q.variant & 8) && wlActive(c))
            return fail(SC_ERR_UNSUPPORTED, "the warp-per-cell kernel (variant bit 3) does not run Wang-Landau moves");
        if (p.transmx > 0) q.transmx = p.transmx;
        if (p.rot_angle > 0) q.rot_angle = p.rot_angle;
        q.chainprob = p.chainprob;
        if (p.chainmmx > 0) q.chainmmx = p.chainmmx;
        if (p.chain_angle > 0) q.chain_angle = p.chain_angle;
        if ((rc = prepareSystem(c, q, npt))) return rc;
    }
    b.stream = b.sys[0]->stream;
    b.device = b.sys[0]->device;
    if (!b.dLadder) {
        if ((rc = b.alloc((void**)&b.dLadder, sizeof(int) * nrep))) return rc;
        if ((rc = b.alloc((void**)&b.dLadderStart, sizeof(int) * R->ladderStartHost.size()))) return rc;
        if ((rc = b.alloc((void**)&b.dExCtr, sizeof(unsigned long long) * (1 + 2 * nrep)))) return rc;
        cudaMemcpy(b.dLadder, R->ladderHost.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice);
        cudaMemcpy(b.dLadderStart, R->ladderStartHost.data(), sizeof(int) * R->ladderStartHost.size(), cudaMemcpyHostToDevice);
        cudaMemset(b.dExCtr, 0, sizeof(unsigned long long) * (1 + 2 * nrep));
        b.nLadders = (int)R->ladderStartHost.size() - 1;
    } else {
        // keep the temperatures the exchanges produced
        std::vector<SweepArgs> cur(nrep);
        cudaMemcpy(cur.data(), b.dArgs, sizeof(SweepArgs) * nrep, cudaMemcpyDeviceToHost);
        for (int k = 0; k < nrep; ++k) b.sys[k]->engine->args.temper = cur[k].temper;
    }
    if ((rc = uploadArgs(b))) return rc;
    RunOut out;
    rc = runBatch(b, p, p.nsweeps, exchangeEvery, p.seed ^ 0xA5A5A5A5ull, out);
    for (int k = 0; k < nrep; ++k) {     // the device's particle vectors (grand-canonical moves)
        const int rcG = finishGrand(b.sys[k], b.dArgs + k);
        if (!rc) rc = rcG;
    }
    if (rc) return rc;
    std::vector<SweepArgs> cur(nrep);
    cudaMemcpy(cur.data(), b.dArgs, sizeof(SweepArgs) * nrep, cudaMemcpyDeviceToHost);
    for (int k = 0; k < nrep; ++k) {
        sc_run_stats s1;
        std::memset(&s1, 0, sizeof s1);
        collectStats(b.sys[k], s1);
        st.moves += s1.moves;
        st.acc_trans += s1.acc_trans; st.rej_trans += s1.rej_trans;
        st.acc_rot += s1.acc_rot; st.rej_rot += s1.rej_rot;
        st.acc_vol += s1.acc_vol; st.rej_vol += s1.rej_vol; st.vol_constrained += s1.vol_constrained;
        st.acc_chain += s1.acc_chain; st.rej_chain += s1.rej_chain;
        st.acc_switch += s1.acc_switch; st.rej_switch += s1.rej_switch;
        st.pairs_tested += s1.pairs_tested; st.pairs_evaluated += s1.pairs_evaluated;
        st.particles += (long)b.sys[k]->conf.p.size();
        if (b.sys[k]->engine->gcOn) {
            GcDev h;
            cudaMemcpy(&h, b.sys[k]->engine->gc, sizeof h, cudaMemcpyDeviceToHost);
            for (int g = 0; g < h.nSpecies; ++g) {
                st.acc_insert += (long)h.ctr[g][1]; st.rej_insert += (long)h.ctr[g][2];
                st.acc_delete += (long)h.ctr[g][3]; st.rej_delete += (long)h.ctr[g][4];
            }
        }
        st.da_stage1_rejected += s1.da_stage1_rejected;
        st.da_stage2_tried += s1.da_stage2_tried;
        st.da_stage2_rejected += s1.da_stage2_rejected;
        st.da_err_rms += s1.da_err_rms * s1.da_err_rms * (double)s1.da_stage2_tried;    // sum of squares for now
        st.da_err_mean += s1.da_err_mean * (double)s1.da_stage2_tried;
        st.energy += s1.energy;
        st.max_drift = std::max(st.max_drift, s1.max_drift);
        if (tempsOut) tempsOut[k] = cur[k].temper;
        if (energiesOut) energiesOut[k] = s1.energy;
        if ((rc = systemErrors(b.sys[k]))) {
            for (Context* c : b.sys) c->engine->energyKnown = false;   // see runSweeps
            return rc;
        }
    }
    if (exTried || exAcc) {
        std::vector<unsigned long long> ctr(1 + 2 * nrep);
        cudaMemcpy(ctr.data(), b.dExCtr, sizeof(unsigned long long) * ctr.size(), cudaMemcpyDeviceToHost);
        for (int k = 0; k < nrep; ++k) {
            if (exTried) exTried[k] = (long)ctr[1 + 2 * k];
            if (exAcc) exAcc[k] = (long)ctr[2 + 2 * k];
        }
    }
    if (st.da_stage2_tried > 0) {
        st.da_err_rms = std::sqrt(st.da_err_rms / (double)st.da_stage2_tried);
        st.da_err_mean /= (double)st.da_stage2_tried;
    }
    st.sweeps = out.sweeps;
    st.seconds = out.seconds;
    st.phase_seconds = out.phaseSeconds;
    st.phase_launches = out.phaseLaunches;
    st.launches = out.launches;
    return SC_OK;
}

}  // namespace scg
