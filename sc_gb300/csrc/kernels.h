// kernels.h -- device state and kernel launchers of the GPU path.
#pragma once

#include <cuda_runtime.h>

#include "sc_common.h"

namespace scg {

// Particle state in HBM, structure of arrays (see pair_energy.cuh for the field layout).
struct DevState {
    double4_32a* pos;      // x, y, z box fractions; w = compact type index
    double4_32a* dir;
    PatchSet* patch;
    int4* mol;         // molecule type, position in molecule, molecule size, first particle of the molecule
    double* box;       // 3 doubles, device resident (volume moves change it on the device)
    int n;
};

struct DevTables {
    const PairParam* params;   // ntypes x ntypes
    const MolParam* mols;
    int ntypes;
    double sqmaxcut;
};

// Trial state of one particle (used by the one-particle trial energy calls).
struct TrialSlot {
    double4_32a pos;
    double4_32a dir;
    PatchSet patch;
};

// Batched PairE(i[k], j[k], conlist(i[k])); energies, verdict bits and segment distance^2.
cudaError_t launchPairBatch(const DevState& s, const DevTables& t, int npairs, const int* I, const int* J, double* E,
                            unsigned* bits, double* dsq, cudaStream_t st);
// oneToAllTrial semantics for a list of targets; trial != nullptr replaces target[0]'s state.
cudaError_t launchOneToAll(const DevState& s, const DevTables& t, int ntargets, const int* targets,
                           const TrialSlot* trial, double* out, cudaStream_t st);
// allToAll over all pairs i > j with conlist(i); per-block partial sums then a deterministic final sum.
cudaError_t launchAllToAll(const DevState& s, const DevTables& t, const double* boxOverride, double* partial,
                           int npartial, double* out, cudaStream_t st);
int allToAllBlocks(int n);
// Updater::alignmentOrder: sum of axis dot products over pairs closer than 1.5.
cudaError_t launchAlignment(const DevState& s, double* partial, int npartial, double* out, cudaStream_t st);
// Count and second-moment sums (xx, yy, zz, xy, xz, yz) of the spherocylinders' axes (7 doubles).
cudaError_t launchAxisMoments(const DevState& s, const DevTables& t, double* out, cudaStream_t st);
// mol2othersTrial: molecule [first, first+size) against the rest with an empty conlist.
cudaError_t launchMolToOthers(const DevState& s, const DevTables& t, int first, int size, double* out, cudaStream_t st);

}  // namespace scg
