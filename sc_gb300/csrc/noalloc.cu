// noalloc.cu -- one-particle energies without any device allocation.
//
// sc_one_to_all allocates (and grows) a scratch buffer with cudaMalloc for the
// target list and the results.  Some callers cannot allow that: code that runs while
// another component owns all free device memory through its own caching allocator
// (a cudaMalloc would fail with out-of-memory there), and code on a latency-critical
// path where cudaMalloc / cudaFree would synchronise the whole device.  For them,
// sc_one_to_all_noalloc stages targets and results in a fixed array compiled into
// the library instead.
//
// The array below is a file-scope device variable: every GPU that loads this library
// holds its 192 KiB until the process exits, and every call on that GPU shares it.
// It is not safe to have two calls in flight on the GPU at once (two contexts on
// different streams, or two host threads): they would overwrite each other's targets
// and results.  The array keeps the previous call's contents; the result region is
// cleared before each use.

#include <mutex>

#include "sc_context.h"

namespace scg {

namespace {

constexpr int kNoallocMaxTargets = SC_NOALLOC_MAX_TARGETS;
constexpr size_t kTargetsBytes = sizeof(int) * kNoallocMaxTargets;
constexpr size_t kScratchBytes = kTargetsBytes + sizeof(double) * kNoallocMaxTargets;

// Targets (int) followed by results (double); 16384 * 12 B = 192 KiB.
static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noallocMutex;
void* g_noallocAddr[kMaxDevices] = {};

}  // namespace

// Device address of the array on `device`.  In host code the name g_noallocScratch only
// denotes a host-side stand-in, never a device address, so the address is looked up with
// that device current and cached.  CUDA loads a module lazily: this lookup is what loads
// the array's module (and commits its memory) on the device, so it runs inside the first
// allocating call on the device (Context::ensureDevice), never inside the no-alloc call.
int noallocLookup(int device) {
    if (device < 0 || device >= kMaxDevices) return fail(SC_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (g_noallocAddr[device]) return SC_OK;
    DeviceScope dev(device);
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess) return cudaFail(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_noallocAddr[device] = p;
    return SC_OK;
}

void* noallocCached(int device) {
    if (device < 0 || device >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    return g_noallocAddr[device];
}

}  // namespace scg

using namespace scg;

extern "C" int sc_one_to_all_noalloc(sc_context* ctx, int ntargets, const int* targets, double* out) {
    if (!ctx || ntargets < 0 || (ntargets > 0 && (!targets || !out))) return fail(SC_ERR_ARG, "null argument");
    Context* c = reinterpret_cast<Context*>(ctx);
    // the copies and the launch go to c->stream, which belongs to c->device
    DeviceScope dev(c->device);
    if (ntargets > kNoallocMaxTargets)
        return fail(SC_ERR_RANGE, "sc_one_to_all_noalloc takes at most " + std::to_string(kNoallocMaxTargets) +
                                      " targets per call");
    int n = (int)c->conf.p.size();
    for (int k = 0; k < ntargets; ++k)
        if (targets[k] < 0 || targets[k] >= n) return fail(SC_ERR_ARG, "target out of range");
    if (!c->devReady || c->hostNewer)
        return fail(SC_ERR_STATE, "the particle state is not on the device: make one allocating call "
                                  "(e.g. sc_one_to_all) after changing it, then use the no-alloc variant");
    if (ntargets == 0) return SC_OK;
    void* base = noallocCached(c->device);
    if (!base)
        return fail(SC_ERR_STATE, "the no-alloc array of this device is not set up: make one allocating call "
                                  "(e.g. sc_one_to_all) on the device first");
    int* dT = (int*)base;
    double* dO = (double*)((unsigned char*)base + kTargetsBytes);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(dT, targets, sizeof(int) * ntargets, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess)
        return cudaFail(e, "copy targets");
    if ((e = cudaMemsetAsync(dO, 0, sizeof(double) * ntargets, c->stream)) != cudaSuccess) return cudaFail(e, "clear results");
    if ((e = launchOneToAll(c->d, c->tables, ntargets, dT, nullptr, dO, c->stream)) != cudaSuccess)
        return cudaFail(e, "one-to-all kernel");
    if ((e = cudaMemcpyAsync(out, dO, sizeof(double) * ntargets, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess)
        return cudaFail(e, "copy results");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "one-to-all (no-alloc)");
    return SC_OK;
}
