// wanglandau.h -- Wang-Landau flat-histogram sampling on the GPU move loop.
//
// The reference's WangLandau class (scOOP/mc/wanglandau.h:16-690, wanglandau.cpp) biases
// every move by weights of one or two order parameters and lowers the weight of the
// visited bin by alpha after every move (accept / reject, wanglandau.h:262-290); alpha is
// halved when the histogram is flat (update, :66-120).  This library supports the order
// parameters whose value only the moves of particles 0 and 1, of the particles near
// particle 0, and the box change:
//   1  z of particle 0 relative to the system's volume-weighted centre   (zOrder,  :551-554)
//   3  z component of particle 0's axis                                  (zOrient, :321-324)
//   4  xy distance of particles 0 and 1                                  (twoPartDist, :395-398)
//   7  particles of type wlmtype within sqrt(WL_CONTACTS) of particle 0  (contParticlesAll,
//      :603-676): only moves of particles within that distance of particle 0's cell change it
//   8  box length in x, 9 box length in y                                (boxSize_x/_y, :376-382)
//
// Weights are kept as w[i] = base[i] - alpha * (hist[i] - hist0[i]): base and hist0 are
// set when alpha changes, hist counts visits as the reference's histogram does, so the
// weight decrements of all moves are integer counts (exact, independent of the order in
// which concurrent updates land).  The table (alpha, weights, histogram) can be shared by
// several walkers -- the reference's multiple walkers, which share weights and histogram
// through MPI shared-memory windows (wanglandau.cpp:184-218) -- while each walker keeps its
// own bins and system centre.
#pragma once

#include <cuda_runtime.h>

namespace scg {

constexpr double kWlGerr = 0.0001;        // WL_GERR     scOOP/structures/macros.h:103
constexpr double kWlAlphaTol = 1.0e-8;    // WL_ALPHATOL macros.h:104
constexpr long kWlMinHist = 1000;         // WL_MINHIST  macros.h:105
constexpr int kWlUpdateEvery = 1000;      // sweeps between flatness checks, updater.cpp:255
constexpr double kWlContacts = 36.0;      // WL_CONTACTS macros.h:107 (squared contact distance)

// Weights and histogram, shared by the walkers of one Wang-Landau run.
struct WlTable {
    double alpha;
    long long updates;       // alpha halvings so far
    int converged;           // update() found a flat histogram with alpha below tolerance
    int pad_;
    double* base;            // weights when alpha last changed
    long long* hist;         // histogram (reset when alpha changes)
    long long* hist0;        // histogram when alpha last changed
};

// One walker: its bins, system centre and the table it biases with.
struct WlDev {
    int dim;                 // 1 or 2 order parameters
    int wlm[2];              // order parameter kinds (0: none)
    int len[2];              // bins per dimension (len[1] = 1 for one dimension)
    int part[2];             // particles whose moves change the orders (-1: none)
    int cell[2];             // their cells in the current sweep (written by kAssign)
    int needCM;              // order 1 in use: the system centre is tracked
    int owner;               // this walker runs the table's flatness checks
    double minorder[2], dorder[2];
    double sysvol;           // sum of the particles' Ia_param volumes (Conf::sysvolume)
    double cmK[3];           // sum of volume * anInt(position) when the orders were set up
    double syscm[3];         // volume-weighted centre, box fractions (Conf::syscm)
    long long cur[2];        // current bins
    unsigned long long chainSeen;   // chain-move attempts already counted
    WlTable* tab;            // weights and histogram (device)
    // order 7: the compact type counted (-1: none present), the count now, and the reach in
    // cells (per axis, set at every sweep's start) of the block of cells around particle 0's
    // cell whose particles can come within the contact distance of particle 0 (0: order 7
    // not in use)
    int contactType;
    int useContacts;
    int reach[3];
    int pad7_;
    long long contacts;
};

__host__ __device__ inline double wlWeight(const WlTable& t, long long i) {
    return t.base[i] - t.alpha * (double)(t.hist[i] - t.hist0[i]);
}
__host__ __device__ inline long long wlIndex(const WlDev& w, const long long o[2]) {
    return o[0] + o[1] * (long long)w.len[0];
}
__host__ __device__ inline bool wlInRange(const WlDev& w, const long long o[2]) {
    for (int k = 0; k < w.dim; ++k)
        if (o[k] < 0 || o[k] >= w.len[k]) return false;
    return true;
}

// Order-parameter bins, as the reference computes them (ceil for positions and box
// lengths, floor for the orientation).
__host__ __device__ inline long long wlZOrder(const WlDev& w, int k, double z0, double cmz, double boxz) {
    return (long long)ceil(((z0 - cmz) * boxz - w.minorder[k]) / w.dorder[k]);
}
__host__ __device__ inline long long wlOrientOrder(const WlDev& w, int k, double dirz) {
    return (long long)floor((dirz - w.minorder[k]) / w.dorder[k]);
}
__host__ __device__ inline long long wlDistOrder(const WlDev& w, int k, const double* p0, const double* p1,
                                                 const double* box) {
    // Cuboid::image (geometry.h:110-128): rint is the reference's round-half-even
    double dx = p0[0] - p1[0], dy = p0[1] - p1[1];
    double rx = box[0] * (dx - rint(dx)), ry = box[1] * (dy - rint(dy));
    return (long long)ceil((sqrt(rx * rx + ry * ry) - w.minorder[k]) / w.dorder[k]);
}
__host__ __device__ inline long long wlBoxOrder(const WlDev& w, int k, double edge) {
    return (long long)ceil((edge - w.minorder[k]) / w.dorder[k]);
}
// WangLandau::particlesInContact (wanglandau.h:660-676): minimum image of box fractions
// (anInt, the reference's round-half-even: rint), scaled by the box
__host__ __device__ inline bool wlInContact(const double* a, const double* p0, const double* box) {
    double x = a[0] - p0[0], y = a[1] - p0[1], z = a[2] - p0[2];
    x = box[0] * (x - rint(x));
    y = box[1] * (y - rint(y));
    z = box[2] * (z - rint(z));
    return x * x + y * y + z * z < kWlContacts;
}
// contParticlesOrder (wanglandau.h:652-654)
__host__ __device__ inline long long wlContactOrder(const WlDev& w, int k, long long count) {
    return (long long)ceil(((double)count - w.minorder[k]) / w.dorder[k]);
}

}  // namespace scg
