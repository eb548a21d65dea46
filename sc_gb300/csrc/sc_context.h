// sc_context.h -- host-side state behind one sc_context handle.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/sc_gb300.h"
#include "kernels.h"
#include "sc_input.h"

namespace scg {

struct SweepEngine;   // sweep.cu: device state of the move loop
struct Batch;         // sweep.cu: systems moved together
struct Surrogate;     // surrogate.cu: learned pair-energy surrogate
struct MlpPacked;     // surrogate.cuh: its BF16 weights in mma fragment order
struct WlHost;        // wanglandau.cu: Wang-Landau weights and histogram
struct WlDev;         // wanglandau.h: their device record

constexpr int kMaxGrandSpecies = 8;

struct Context {
    Options opts;
    Topology topo;
    std::string topText;       // the top.init text the context was opened with (top.last)
    Config conf;
    std::vector<MolParam> mols;
    std::vector<int4> molInfo;
    std::vector<int> usedTypes;
    int compactOf[MAXT];

    int device = 0;
    bool devReady = false;
    bool hostNewer = true;    // host copy changed since the last upload
    bool devNewer = false;    // device copy changed (moves) since the last download
    cudaStream_t stream = nullptr;
    std::vector<void*> allocations;
    void* hostStage = nullptr;   // pinned staging of the state copies (positions, axes, patches, box)

    DevState d{};
    DevTables tables{};
    PairParam* dParams = nullptr;
    MolParam* dMols = nullptr;
    TrialSlot* dTrial = nullptr;
    double* dScalars = nullptr;
    double* dPartial = nullptr;
    int nPartial = 0;
    void* dScratch = nullptr;
    size_t scratchBytes = 0;

    int trialTarget = -1;
    Particle trialState;

    Surrogate* surrogate = nullptr;   // first stage of delayed-acceptance moves (not owned)
    WlHost* wl = nullptr;             // Wang-Landau bias (sc_wl_load), owned
    SweepEngine* engine = nullptr;
    Batch* batch = nullptr;
    long lastLaunches = 0;     // kernels launched by the last move loop
    // maximum steps the equilibration adapts (Updater::optimizeStep / optimizeRot, the Disp
    // records of statistics.h:53-66): per particle type, per chain molecule type (the first
    // kMaxChainSteps), and the box edge; the last run's acceptance counts feed them
    struct Disp { double mx = 0.0, oldrmsd = 0.0, oldmx = 0.0; long acc = 0, rej = 0; };
    static constexpr int kMaxChainSteps = 8;
    bool stepsInit = false;
    Disp trans[MAXT], rot[MAXT], chainm[kMaxChainSteps], chainr[kMaxChainSteps], edge;
    double chainAdapted[kMaxChainSteps] = {0};   // chain displacement length per molecule type (0: options)
    long adjustments = 0;
    // sc_tune's choice per mode (index: delayed 0 / 1): stencil reach and kernel variant
    // used by runs that pass variant = -1 (stencil 0 then takes the tuned reach too)
    int tunedStencil[2] = {0, 0};
    int tunedVariant[2] = {-1, -1};
    // grand-canonical species: the molecule types with an ACTIVITY (MoleculeParams::activity,
    // chemPot; moleculeparams.h:43-52), in molecule-type order, with the acceptance record of
    // Statistics::grand (steps, insertions, deletions, the sum of counts after each step)
    struct Grand {
        int molType = 0, type = 0;
        double activity = -1.0, chemPot = -1.0;
        long steps = 0, insAcc = 0, insRej = 0, delAcc = 0, delRej = 0;
        double countSum = 0.0;
    };
    std::vector<Grand> grand;
    int cap = 0;              // particle slots of the device state arrays (>= the particle count)
    // type switching (MoveCreator::switchTypeMove): per molecule type and position in the
    // molecule (MAXCHL each) the compact type, the compact switch type (-1: none) and delta_mu
    // as the move reads it, an int (movecreator.cpp:238-243)
    std::vector<int4> switchTab;
    int4* dSwitch = nullptr;
    bool anySwitch = false;   // some molecule type has a switch type

    Context() = default;
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    ~Context();

    int setup(std::string& err);
    void rebuildMolInfo();
    int ensureDevice();
    int uploadState();
    int downloadState();
    int allocDev(void** p, size_t bytes);
    int grow(int newCap);     // state arrays of newCap slots, keeping the first d.n particles
    int scratch(size_t bytes);
    void freeDevice();
    PairParam devParam(int t1, int t2) const;
};

// Makes a context's device the calling thread's current device for the lifetime of the
// scope and gives the caller's device back afterwards, so that every copy and launch of
// an entry point goes to the device (and the stream) the context lives on, whatever
// device the calling thread had selected.  Without a usable CUDA device it does nothing.
struct DeviceScope {
    int prev = -1;
    int want = -1;
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) { prev = -1; cudaGetLastError(); return; }
        want = device;
        if (prev != device && cudaSetDevice(device) != cudaSuccess) { want = prev; cudaGetLastError(); }
    }
    ~DeviceScope() {
        if (prev >= 0 && want != prev) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

int fail(int code, const std::string& msg);
// Device address of the no-allocation entry point's fixed array on `device` (noalloc.cu).
// Looked up by the first allocating call on the device (Context::ensureDevice), because
// the lookup loads the array's module, which may allocate; afterwards it only reads a cache.
int noallocLookup(int device);
void* noallocCached(int device);
const MlpPacked* surrogatePacked(const Surrogate* s);
float surrogateCutoff(const Surrogate* s);
float surrogateRange(Context* c);
int cudaFail(cudaError_t e, const char* where);
int runSweeps(Context* c, const sc_run_params& p, sc_run_stats& st);
int adjustSteps(Context* c);
void initStepSizes(Context* c);      // the Disp records from the options (once)
int equilibrate(Context* c, const sc_run_params& p, long nequil, long adjust, sc_run_stats& st);
int tuneSweeps(Context* c, const sc_run_params& p, int sweeps, sc_run_params& best, double* rates, int* ncand);
int screenSurvivors(Context* c, int ntargets, const int* targets, long cap, int* I, int* J, unsigned char* B,
                    long* count);
void destroyEngine(Context* c);
int createReplicas(Context* const* sys, int nrep, const double* temps, const int* group, void** out);
void destroyReplicas(void* h);
int runReplicas(void* h, const sc_run_params& p, int exchangeEvery, sc_run_stats& st, double* tempsOut,
                double* energiesOut, long* exTried, long* exAcc);
// Wang-Landau (wanglandau.cu)
bool wlActive(const Context* c);                      // weights loaded and options wlm > 0
int wlCheckRun(const Context* c, const sc_run_params& p);
int wlPrepare(Context* c, bool hostChanged);          // device record current before a run
WlDev* wlDevice(const Context* c);                    // nullptr when inactive
bool wlConverged(Context* c);                         // reads the device flag (stream synchronised)
void destroyWl(Context* c);

}  // namespace scg
