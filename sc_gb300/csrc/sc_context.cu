// sc_context.cu -- the C ABI (include/sc_gb300.h): context set-up, host<->device state
// and the energy entry points.  The move loop lives in sweep.cu.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sc_gb300.h"
#include "kernels.h"
#include "host_parallel.h"
#include "sc_context.h"

namespace scg {

thread_local std::string g_lastError;

int fail(int code, const std::string& msg) {
    g_lastError = msg;
    return code;
}

int cudaFail(cudaError_t e, const char* where) {
    return fail(SC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

Context::~Context() { freeDevice(); }

void Context::freeDevice() {
    destroyEngine(this);
    destroyWl(this);
    if (!devReady) return;
    DeviceScope dev(device);
    for (void* p : allocations) cudaFree(p);
    allocations.clear();
    if (hostStage) cudaFreeHost(hostStage);
    hostStage = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
    devReady = false;
}

int Context::allocDev(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) return cudaFail(e, "cudaMalloc");
    allocations.push_back(*p);
    return SC_OK;
}

PairParam Context::devParam(int t1, int t2) const {
    const IaParam& s = topo.ia[t1][t2];
    PairParam p;
    std::memset(&p, 0, sizeof p);
    int g0 = s.geotype[0], g1 = s.geotype[1];
    p.geotype[0] = g0;
    p.geotype[1] = g1;
    p.kind = functorKind(g0, g1);
    p.exclude = s.exclude ? 1 : 0;
    // getGeoTypes of the selected functor (paire.h:486-497, 674-685, 891-906)
    if (p.kind == K_SC_PSC) {
        p.fCH = (g0 == CHPSC || g0 == TCHPSC); p.sCH = (g1 == CHPSC || g1 == TCHPSC);
        p.fT = (g0 == TPSC || g0 == TCHPSC); p.sT = (g1 == TPSC || g1 == TCHPSC);
        p.firstPsc = p.secondPsc = 1;
    } else if (p.kind == K_SC_CPSC) {
        p.fCH = (g0 == CHCPSC || g0 == TCHCPSC); p.sCH = (g1 == CHCPSC || g1 == TCHCPSC);
        p.fT = (g0 == TCPSC || g0 == TCHCPSC); p.sT = (g1 == TCPSC || g1 == TCHCPSC);
    } else if (p.kind == K_SC_PSC_CPSC) {
        p.fCH = isChiral(g0); p.sCH = isChiral(g1); p.fT = isTwoPatch(g0); p.sT = isTwoPatch(g1);
        p.firstPsc = isPscFamily(g0);
        p.secondPsc = !p.firstPsc;
    }
    // PscSpa / CPscSpa::getGeoTypes (paire.h:981-1005), read from the entry with the SC first
    if (g0 < SP && p.kind == K_MIX_PSC_SP) { p.mixChiral = (g0 == CHPSC || g0 == TCHPSC); p.mixSec = (g0 == TPSC || g0 == TCHPSC); }
    if (g0 < SP && p.kind == K_MIX_CPSC_SP) { p.mixChiral = (g0 == CHCPSC || g0 == TCHCPSC); p.mixSec = (g0 == TCPSC || g0 == TCHCPSC); }
    p.sigma = s.sigma; p.epsilon = s.epsilon; p.A = s.A; p.B = s.B; p.pdis = s.pdis; p.pswitch = s.pswitch;
    p.pswitchINV = s.pswitchINV;
    for (int k = 0; k < 4; ++k) { p.pcangl[k] = s.pcangl[k]; p.pcanglsw[k] = s.pcanglsw[k]; }
    p.rcut = s.rcut; p.rcutSq = s.rcutSq; p.rcutwca = s.rcutwca; p.rcutwcaSq = s.rcutwcaSq;
    p.half_len[0] = s.half_len[0]; p.half_len[1] = s.half_len[1];
    p.parallel = s.parallel;
    // beyond these distances the repulsive and attractive branches are both off
    // (SpheroCylinder::operator() paire.h:1130-1137, MixSpSc::operator() paire.h:1036-1041)
    if (p.kind >= K_SC_PSC_CPSC && p.kind <= K_SC_SCA) {
        p.screen = 1;
        p.screenSq = (s.epsilon == 0.0 || s.exclude) ? s.rcutwcaSq : std::max(s.rcutSq, s.rcutwcaSq);
    } else if (p.kind >= K_MIX_SCA_SPA) {
        const IaParam& q = (g0 < SP) ? s : topo.ia[t2][t1];
        p.screen = 2;
        p.scFirst = g0 < SP;
        p.scHalf = q.half_len[0];
        p.screenSq = (q.epsilon == 0.0 || q.exclude) ? q.rcutwcaSq : std::max(q.rcutSq, q.rcutwcaSq);
    } else if (p.kind == K_NONE) {
        p.screen = 3;
    }
    p.simple = (p.kind == K_SC_PSC_CPSC || p.kind == K_SC_CPSC || p.kind == K_SC_PSC);   // patchy SC-SC
    return p;
}

int Context::setup(std::string& err) {
    // compact type indices for the device table
    std::memset(compactOf, -1, sizeof compactOf);
    usedTypes.clear();
    for (int t = 0; t < MAXT; ++t)
        if (topo.ia[t][t].geotype[0] != 0) {
            compactOf[t] = (int)usedTypes.size();
            usedTypes.push_back(t);
        }
    if ((int)usedTypes.size() > MAX_DEV_TYPES) { err = "more particle types than the device table holds (16)"; return SC_ERR_RANGE; }
    // molecule records
    mols.clear();
    for (auto& m : topo.mols) {
        MolParam mp;
        std::memset(&mp, 0, sizeof mp);
        mp.size = (int)m.types.size();
        // ParticleVector::getConlist (Conf.h:97-146): the last defined bond kind wins
        if (m.bond1c >= 0.0 || m.bonddc >= 0.0 || m.bondhc >= 0.0) {
            mp.bonded = 1;
            if (m.bond1c >= 0.0) { mp.eq0 = m.bond1eq; mp.c0 = m.bond1c; mp.mod0 = 0; mp.mod1 = 0; mp.sp = 0; }
            if (m.bonddc >= 0.0) { mp.eq0 = 0.0; mp.c0 = m.bonddc; mp.mod0 = m.bonddeq; mp.mod1 = 0; mp.sp = 0; }
            if (m.bondhc >= 0.0) { mp.eq0 = 0.0; mp.c0 = m.bondhc; mp.mod0 = m.bondheq; mp.mod1 = m.bondheq; mp.sp = m.bondheq; }
        }
        if (m.bond2c >= 0.0) { mp.bonded2 = 1; mp.eq1 = m.bond2eq; mp.c1 = m.bond2c; }
        mp.angle1c = m.angle1c; mp.angle1eq = m.angle1eq; mp.angle2c = m.angle2c; mp.angle2eq = m.angle2eq;
        mols.push_back(mp);
    }
    if (mols.empty()) { MolParam z; std::memset(&z, 0, sizeof z); z.size = 1; mols.push_back(z); }
    rebuildMolInfo();
    // switch types (setParticlesParams / initSwitchList, inicializer.cpp:60-87, 428-431)
    switchTab.assign(mols.size() * MAXCHL, make_int4(-1, -1, 0, 0));
    anySwitch = false;
    for (size_t m = 0; m < topo.mols.size(); ++m)
        for (size_t k = 0; k < topo.mols[m].types.size(); ++k) {
            const int sw = topo.mols[m].switchTypes[k];
            switchTab[m * MAXCHL + k] = make_int4(compactOf[topo.mols[m].types[k]], sw >= 0 ? compactOf[sw] : -1,
                                                  (int)topo.mols[m].deltaMu[k], 0);
            anySwitch |= sw >= 0;
        }
    // grand-canonical species (inicializer.cpp:36-47, 1087-1096; main.cpp:104-108, 128-139)
    grand.clear();
    int firstGrand = -1;
    for (size_t m = 0; m < topo.mols.size(); ++m) {
        if (topo.mols[m].activity == -1.0) continue;
        if (opts.nGrandCanon == 0) { err = "Activity stated in top.init, But nGrandCanon=0 in options"; return SC_ERR_PARSE; }
        if (topo.mols[m].types.size() != 1) {
            err = "grand-canonical insertion of chains draws from a [Pool] configuration, which is outside the GPU path";
            return SC_ERR_UNSUPPORTED;
        }
        Grand g;
        g.molType = (int)m;
        g.type = topo.mols[m].types[0];
        g.activity = topo.mols[m].activity;
        g.chemPot = std::log(g.activity * 6.022137e23 * 1e-24);   // Nav of inicializer.cpp:934
        grand.push_back(g);
        if (firstGrand < 0) firstGrand = (int)m;
    }
    if (opts.nGrandCanon != 0 && grand.empty()) {
        err = "In options nGrandCanon != 0, but no activity set for any species in top.init";
        return SC_ERR_PARSE;
    }
    if ((int)grand.size() > kMaxGrandSpecies) { err = "more than 8 grand-canonical species"; return SC_ERR_RANGE; }
    // an insertion or deletion moves the particles behind it by one slot: only single
    // particles may sit there (no bond partner index changes)
    for (size_t m = firstGrand < 0 ? topo.mols.size() : (size_t)firstGrand; m < topo.mols.size(); ++m)
        if (topo.mols[m].types.size() != 1) {
            err = "the molecule types from the first grand-canonical species on must be single particles "
                  "(list the grand-canonical species last)";
            return SC_ERR_UNSUPPORTED;
        }
    return SC_OK;
}

// Molecule record of every particle: its type, position in the molecule, the molecule's
// size and first particle (ParticleVector::first and the molecule sizes).
void Context::rebuildMolInfo() {
    molInfo.resize(conf.p.size());
    for (size_t i = 0; i < conf.p.size(); ++i) {
        int m = conf.p[i].molType;
        int size = (int)topo.mols[m].types.size();
        int pos = ((int)i - conf.first[m]) % size;
        molInfo[i] = make_int4(m, pos, size, (int)i - pos);
    }
}

int Context::ensureDevice() {
    // every call: the stream and the buffers below belong to `device` (the entry points
    // hold a DeviceScope that gives the caller's device back when they return)
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cudaFail(e, "cudaSetDevice");
    if (!devReady) {
        // the no-allocation entry point's array: its address lookup loads the module that
        // holds it, which may allocate, so it is done here, in an allocating call
        int rc0 = noallocLookup(device);
        if (rc0) return rc0;
        e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cudaFail(e, "cudaStreamCreate");
        int n = (int)conf.p.size();
        int T = (int)usedTypes.size();
        int rc;
        // grand-canonical systems keep free slots for insertions (grown on demand by the
        // move loop, Context::grow)
        cap = grand.empty() ? n : n + std::max(256, n / 2);
        const size_t slots = (size_t)std::max(cap, 1);
        if ((rc = allocDev((void**)&d.pos, sizeof(double4_32a) * slots))) return rc;
        if ((rc = allocDev((void**)&d.dir, sizeof(double4_32a) * slots))) return rc;
        if ((rc = allocDev((void**)&d.patch, sizeof(PatchSet) * slots))) return rc;
        if ((rc = allocDev((void**)&d.mol, sizeof(int4) * slots))) return rc;
        if ((rc = allocDev((void**)&d.box, sizeof(double) * 4))) return rc;
        if ((rc = allocDev((void**)&dParams, sizeof(PairParam) * T * T))) return rc;
        if ((rc = allocDev((void**)&dMols, sizeof(MolParam) * mols.size()))) return rc;
        if ((rc = allocDev((void**)&dTrial, sizeof(TrialSlot)))) return rc;
        if ((rc = allocDev((void**)&dScalars, sizeof(double) * 64))) return rc;
        if ((rc = allocDev((void**)&dSwitch, sizeof(int4) * switchTab.size()))) return rc;
        e = cudaMemcpy(dSwitch, switchTab.data(), sizeof(int4) * switchTab.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cudaFail(e, "upload switch types");
        nPartial = allToAllBlocks((int)slots) + 1;
        if ((rc = allocDev((void**)&dPartial, sizeof(double) * nPartial))) return rc;
        d.n = n;
        e = cudaMallocHost(&hostStage, (sizeof(double4_32a) * 2 + sizeof(PatchSet)) * slots + 64);
        if (e != cudaSuccess) { hostStage = nullptr; return cudaFail(e, "cudaMallocHost (state staging)"); }
        std::vector<PairParam> hp(T * T);
        for (int a = 0; a < T; ++a)
            for (int b = 0; b < T; ++b) hp[a * T + b] = devParam(usedTypes[a], usedTypes[b]);
        e = cudaMemcpy(dParams, hp.data(), sizeof(PairParam) * T * T, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cudaFail(e, "upload params");
        e = cudaMemcpy(dMols, mols.data(), sizeof(MolParam) * mols.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cudaFail(e, "upload molecules");
        e = cudaMemcpy(d.mol, molInfo.data(), sizeof(int4) * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cudaFail(e, "upload molecule records");
        tables.params = dParams;
        tables.mols = dMols;
        tables.ntypes = T;
        tables.sqmaxcut = topo.sqmaxcut;
        devReady = true;
        hostNewer = true;
    }
    if (hostNewer) {
        int rc = uploadState();
        if (rc) return rc;
    }
    return SC_OK;
}

// Moves the device state into arrays of newCap slots, keeping the first d.n particles (the
// grand-canonical moves fill the free slots; the caller has synchronised the stream).
int Context::grow(int newCap) {
    if (newCap <= cap) return SC_OK;
    DeviceScope dev(device);
    const size_t slots = (size_t)newCap;
    const size_t n = (size_t)d.n;
    auto replace = [&](void** p, size_t elem) -> int {
        void* q = nullptr;
        int rc = allocDev(&q, elem * slots);
        if (rc) return rc;
        cudaError_t e = cudaMemcpy(q, *p, elem * n, cudaMemcpyDeviceToDevice);
        if (e != cudaSuccess) return cudaFail(e, "grow state");
        cudaFree(*p);
        allocations.erase(std::find(allocations.begin(), allocations.end(), *p));
        *p = q;
        return SC_OK;
    };
    int rc;
    if ((rc = replace((void**)&d.pos, sizeof(double4_32a)))) return rc;
    if ((rc = replace((void**)&d.dir, sizeof(double4_32a)))) return rc;
    if ((rc = replace((void**)&d.patch, sizeof(PatchSet)))) return rc;
    if ((rc = replace((void**)&d.mol, sizeof(int4)))) return rc;
    const int np = allToAllBlocks(newCap) + 1;
    if (np > nPartial) {
        cudaFree(dPartial);
        allocations.erase(std::find(allocations.begin(), allocations.end(), (void*)dPartial));
        dPartial = nullptr;
        if ((rc = allocDev((void**)&dPartial, sizeof(double) * np))) return rc;
        nPartial = np;
    }
    void* stage = nullptr;
    cudaError_t e = cudaMallocHost(&stage, (sizeof(double4_32a) * 2 + sizeof(PatchSet)) * slots + 64);
    if (e != cudaSuccess) return cudaFail(e, "cudaMallocHost (state staging)");
    cudaFreeHost(hostStage);
    hostStage = stage;
    cap = newCap;
    return SC_OK;
}

int Context::uploadState() {
    int n = (int)conf.p.size();
    if (n > cap) {                 // a grand-canonical vector longer than the slots
        int rc = grow(n + std::max(256, n / 2));
        if (rc) return rc;
    }
    d.n = n;
    // the state goes through one pinned staging block, so the copies are true DMA
    double* box = (double*)hostStage;
    double4_32a* hp = (double4_32a*)((char*)hostStage + 64);
    double4_32a* hd = hp + n;
    PatchSet* hs = (PatchSet*)(hd + n);
    parallelRange(n, [&](int lo, int hi) {
        for (int i = lo; i < hi; ++i) {
            const Particle& p = conf.p[i];
            hp[i] = make_double4_32a(p.pos.x, p.pos.y, p.pos.z, (double)compactOf[p.type]);
            hd[i] = make_double4_32a(p.dir.x, p.dir.y, p.dir.z, (double)p.switched);   // w: switched
            PatchSet& s = hs[i];
            for (int k = 0; k < 2; ++k) { s.pd[k][0] = p.pd[k].x; s.pd[k][1] = p.pd[k].y; s.pd[k][2] = p.pd[k].z; }
            for (int k = 0; k < 4; ++k) { s.ps[k][0] = p.ps[k].x; s.ps[k][1] = p.ps[k].y; s.ps[k][2] = p.ps[k].z; }
            for (int k = 0; k < 2; ++k) { s.ch[k][0] = p.ch[k].x; s.ch[k][1] = p.ch[k].y; s.ch[k][2] = p.ch[k].z; }
        }
    });
    box[0] = conf.box.x; box[1] = conf.box.y; box[2] = conf.box.z; box[3] = 0.0;
    cudaError_t e;
    // grand-canonical moves reorder the molecule records on the device: the host's go up too
    if (!grand.empty() && n > 0 &&
        (e = cudaMemcpyAsync(d.mol, molInfo.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
        return cudaFail(e, "upload molecule records");
    if ((e = cudaMemcpyAsync(d.pos, hp, sizeof(double4_32a) * n, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return cudaFail(e, "upload pos");
    if ((e = cudaMemcpyAsync(d.dir, hd, sizeof(double4_32a) * n, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return cudaFail(e, "upload dir");
    if ((e = cudaMemcpyAsync(d.patch, hs, sizeof(PatchSet) * n, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return cudaFail(e, "upload patch");
    if ((e = cudaMemcpyAsync(d.box, box, sizeof(double) * 4, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return cudaFail(e, "upload box");
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cudaFail(e, "upload sync");
    hostNewer = false;
    return SC_OK;
}

int Context::downloadState() {
    if (!devReady || !devNewer) return SC_OK;
    DeviceScope dev(device);
    int n = (int)conf.p.size();
    double* box = (double*)hostStage;
    double4_32a* hp = (double4_32a*)((char*)hostStage + 64);
    double4_32a* hd = hp + n;
    PatchSet* hs = (PatchSet*)(hd + n);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(hp, d.pos, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return cudaFail(e, "download pos");
    if ((e = cudaMemcpyAsync(hd, d.dir, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return cudaFail(e, "download dir");
    if ((e = cudaMemcpyAsync(hs, d.patch, sizeof(PatchSet) * n, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return cudaFail(e, "download patch");
    if ((e = cudaMemcpyAsync(box, d.box, sizeof(double) * 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return cudaFail(e, "download box");
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cudaFail(e, "download sync");
    parallelRange(n, [&](int lo, int hi) {
        for (int i = lo; i < hi; ++i) {
            Particle& p = conf.p[i];
            p.pos = {hp[i].x, hp[i].y, hp[i].z};
            p.dir = {hd[i].x, hd[i].y, hd[i].z};
            const int ct = (int)hp[i].w;      // compact type (inserted and switched particles change it)
            if (ct >= 0 && ct < (int)usedTypes.size()) p.type = usedTypes[ct];
            p.switched = (int)hd[i].w;
            const PatchSet& s = hs[i];
            for (int k = 0; k < 2; ++k) p.pd[k] = {s.pd[k][0], s.pd[k][1], s.pd[k][2]};
            for (int k = 0; k < 4; ++k) p.ps[k] = {s.ps[k][0], s.ps[k][1], s.ps[k][2]};
            for (int k = 0; k < 2; ++k) p.ch[k] = {s.ch[k][0], s.ch[k][1], s.ch[k][2]};
        }
    });
    conf.box = {box[0], box[1], box[2]};
    devNewer = false;
    return SC_OK;
}

int Context::scratch(size_t bytes) {
    if (bytes <= scratchBytes) return SC_OK;
    if (dScratch) {
        cudaFree(dScratch);
        for (auto it = allocations.begin(); it != allocations.end(); ++it)
            if (*it == dScratch) { allocations.erase(it); break; }
        dScratch = nullptr;
    }
    int rc = allocDev(&dScratch, bytes);
    if (rc) return rc;
    scratchBytes = bytes;
    return SC_OK;
}

// Reads the three inputs into a freshly constructed context.
int initContext(Context* c, const std::string& opt, const std::string& top, const std::string& cfg) {
    std::string err;
    int rc;
    if (readOptionsText(opt, c->opts, err)) return fail(SC_ERR_PARSE, err);
    if (readTopologyText(top, c->topo, err)) return fail(err.find("outside") != std::string::npos ? SC_ERR_UNSUPPORTED : SC_ERR_PARSE, err);
    c->topText = top;
    if (buildParticles(c->topo, c->conf, err)) return fail(SC_ERR_PARSE, err);
    if (readConfigText(cfg, c->topo, c->conf, err)) return fail(err.find("outside") != std::string::npos ? SC_ERR_UNSUPPORTED : SC_ERR_PARSE, err);
    partVecInit(c->topo, c->conf);
    if ((rc = c->setup(err))) return fail(rc, err);
    return SC_OK;
}

bool readFile(const char* path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

}  // namespace scg

using namespace scg;

struct sc_context : public Context {};

static Context* C(sc_context* c) { return static_cast<Context*>(c); }
static const Context* C(const sc_context* c) { return static_cast<const Context*>(c); }

extern "C" {

const char* sc_last_error(void) { return g_lastError.c_str(); }
const char* sc_version(void) { return "sc_gb300 0.1 (sm_103a)"; }

int sc_open_text(const char* options, const char* top, const char* config, sc_context** out) {
    if (!options || !top || !config || !out) return fail(SC_ERR_ARG, "null argument");
    sc_context* h = new sc_context();
    int rc = initContext(h, options, top, config);
    if (rc) { delete h; return rc; }
    *out = h;
    return SC_OK;
}

int sc_open(const char* options_path, const char* top_path, const char* config_path, sc_context** out) {
    if (!options_path || !top_path || !config_path || !out) return fail(SC_ERR_ARG, "null argument");
    std::string o, t, c;
    if (!readFile(options_path, o)) return fail(SC_ERR_IO, std::string("cannot read ") + options_path);
    if (!readFile(top_path, t)) return fail(SC_ERR_IO, std::string("cannot read ") + top_path);
    if (!readFile(config_path, c)) return fail(SC_ERR_IO, std::string("cannot read ") + config_path);
    int rc = sc_open_text(o.c_str(), t.c_str(), c.c_str(), out);
    if (rc || C(*out)->opts.wlm[0] <= 0) return rc;
    // the reference reads its Wang-Landau weights from wl.dat (structures.h:93, updater.h:19)
    std::string dir = options_path;
    size_t slash = dir.find_last_of('/');
    std::string wl = (slash == std::string::npos ? std::string() : dir.substr(0, slash + 1)) + "wl.dat";
    std::string text;
    if (!readFile(wl.c_str(), text)) return SC_OK;
    if ((rc = sc_wl_load_text(*out, text.c_str()))) {
        sc_close(*out);
        *out = nullptr;
    }
    return rc;
}

int sc_close(sc_context* ctx) {
    if (!ctx) return fail(SC_ERR_ARG, "null context");
    delete ctx;
    return SC_OK;
}

int sc_set_device(sc_context* ctx, int device) {
    if (!ctx) return fail(SC_ERR_ARG, "null context");
    if (C(ctx)->devReady) return fail(SC_ERR_STATE, "device already in use by this context");
    C(ctx)->device = device;
    return SC_OK;
}

int sc_num_particles(const sc_context* ctx, int* n) {
    if (!ctx || !n) return fail(SC_ERR_ARG, "null argument");
    *n = (int)C(ctx)->conf.p.size();
    return SC_OK;
}

int sc_get_box(sc_context* ctx, double box[3]) {
    if (!ctx || !box) return fail(SC_ERR_ARG, "null argument");
    int rc = C(ctx)->downloadState();
    if (rc) return rc;
    box[0] = C(ctx)->conf.box.x; box[1] = C(ctx)->conf.box.y; box[2] = C(ctx)->conf.box.z;
    return SC_OK;
}

int sc_set_box(sc_context* ctx, const double box[3]) {
    if (!ctx || !box) return fail(SC_ERR_ARG, "null argument");
    if (!(box[0] > 0 && box[1] > 0 && box[2] > 0)) return fail(SC_ERR_ARG, "box edges must be positive");
    int rc = C(ctx)->downloadState();
    if (rc) return rc;
    C(ctx)->conf.box = {box[0], box[1], box[2]};
    C(ctx)->hostNewer = true;
    return SC_OK;
}

int sc_cutoff(const sc_context* ctx, double* sqmaxcut, double* maxcut) {
    if (!ctx) return fail(SC_ERR_ARG, "null context");
    if (sqmaxcut) *sqmaxcut = C(ctx)->topo.sqmaxcut;
    if (maxcut) *maxcut = C(ctx)->topo.maxcut;
    return SC_OK;
}

int sc_get_pair_param(const sc_context* ctx, int t1, int t2, sc_pair_param* out) {
    if (!ctx || !out) return fail(SC_ERR_ARG, "null argument");
    if (t1 < 0 || t2 < 0 || t1 >= MAXT || t2 >= MAXT) return fail(SC_ERR_ARG, "type out of range");
    const IaParam& s = C(ctx)->topo.ia[t1][t2];
    std::memset(out, 0, sizeof *out);
    out->geotype[0] = s.geotype[0]; out->geotype[1] = s.geotype[1];
    out->exclude = s.exclude; out->kind = functorKind(s.geotype[0], s.geotype[1]);
    out->sigma = s.sigma; out->epsilon = s.epsilon; out->A = s.A; out->B = s.B; out->pdis = s.pdis;
    out->pswitch = s.pswitch; out->pswitchINV = s.pswitchINV;
    for (int k = 0; k < 4; ++k) {
        out->pcangl[k] = s.pcangl[k]; out->pcanglsw[k] = s.pcanglsw[k];
        out->pcoshalfi[k] = s.pcoshalfi[k]; out->psinhalfi[k] = s.psinhalfi[k];
    }
    out->rcut = s.rcut; out->rcutSq = s.rcutSq; out->rcutwca = s.rcutwca; out->rcutwcaSq = s.rcutwcaSq;
    for (int k = 0; k < 2; ++k) {
        out->csecpatchrot[k] = s.csecpatchrot[k]; out->ssecpatchrot[k] = s.ssecpatchrot[k];
        out->len[k] = s.len[k]; out->half_len[k] = s.half_len[k];
        out->chiral_cos[k] = s.chiral_cos[k]; out->chiral_sin[k] = s.chiral_sin[k];
    }
    out->volume = s.volume;
    out->parallel = s.parallel;
    return SC_OK;
}

static void toParticle(const Particle& p, sc_particle* o) {
    o->pos[0] = p.pos.x; o->pos[1] = p.pos.y; o->pos[2] = p.pos.z;
    o->dir[0] = p.dir.x; o->dir[1] = p.dir.y; o->dir[2] = p.dir.z;
    for (int k = 0; k < 2; ++k) { o->patchdir[k][0] = p.pd[k].x; o->patchdir[k][1] = p.pd[k].y; o->patchdir[k][2] = p.pd[k].z; }
    for (int k = 0; k < 4; ++k) { o->patchsides[k][0] = p.ps[k].x; o->patchsides[k][1] = p.ps[k].y; o->patchsides[k][2] = p.ps[k].z; }
    for (int k = 0; k < 2; ++k) { o->chdir[k][0] = p.ch[k].x; o->chdir[k][1] = p.ch[k].y; o->chdir[k][2] = p.ch[k].z; }
    o->type = p.type;
    o->molType = p.molType;
}

int sc_get_particles(sc_context* ctx, int first, int count, sc_particle* out) {
    if (!ctx || (!out && count > 0)) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    if (first < 0 || count < 0 || first + count > (int)c->conf.p.size()) return fail(SC_ERR_ARG, "particle range out of bounds");
    int rc = c->downloadState();
    if (rc) return rc;
    parallelRange(count, [&](int lo, int hi) {
        for (int k = lo; k < hi; ++k) toParticle(c->conf.p[first + k], &out[k]);
    });
    return SC_OK;
}

int sc_set_particles(sc_context* ctx, int first, int count, const sc_particle* in) {
    if (!ctx || (!in && count > 0)) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    if (first < 0 || count < 0 || first + count > (int)c->conf.p.size()) return fail(SC_ERR_ARG, "particle range out of bounds");
    int rc = c->downloadState();
    if (rc) return rc;
    // every type is checked before anything is written: a refused call changes nothing
    for (int k = 0; k < count; ++k)
        if (in[k].type != c->conf.p[first + k].type)
            return fail(SC_ERR_ARG, "sc_set_particles cannot change a particle's type");
    parallelRange(count, [&](int lo, int hi) {
        for (int k = lo; k < hi; ++k) {
            Particle& p = c->conf.p[first + k];
            const sc_particle& s = in[k];
            p.pos = {s.pos[0], s.pos[1], s.pos[2]};
            p.dir = {s.dir[0], s.dir[1], s.dir[2]};
            for (int q = 0; q < 2; ++q) p.pd[q] = {s.patchdir[q][0], s.patchdir[q][1], s.patchdir[q][2]};
            for (int q = 0; q < 4; ++q) p.ps[q] = {s.patchsides[q][0], s.patchsides[q][1], s.patchsides[q][2]};
            for (int q = 0; q < 2; ++q) p.ch[q] = {s.chdir[q][0], s.chdir[q][1], s.chdir[q][2]};
        }
    });
    c->hostNewer = true;
    return SC_OK;
}

int sc_write_config(sc_context* ctx, const char* path) {
    if (!ctx || !path) return fail(SC_ERR_ARG, "null argument");
    int rc = C(ctx)->downloadState();
    if (rc) return rc;
    std::string txt = drawConfig(C(ctx)->conf);
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(SC_ERR_IO, std::string("cannot write ") + path);
    std::fwrite(txt.data(), 1, txt.size(), f);
    std::fclose(f);
    return SC_OK;
}

int sc_pair_energies(sc_context* ctx, int npairs, const int* I, const int* J, double* E, unsigned* V, double* D) {
    if (!ctx || npairs < 0 || (npairs > 0 && (!I || !J || !E))) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    int n = (int)c->conf.p.size();
    for (int k = 0; k < npairs; ++k)
        if (I[k] < 0 || J[k] < 0 || I[k] >= n || J[k] >= n) return fail(SC_ERR_ARG, "pair index out of range");
    if (npairs == 0) return SC_OK;
    int rc = c->ensureDevice();
    if (rc) return rc;
    size_t bytes = (size_t)npairs * (2 * sizeof(int) + 2 * sizeof(double) + sizeof(unsigned)) + 256;
    if ((rc = c->scratch(bytes))) return rc;
    char* base = (char*)c->dScratch;
    int* dI = (int*)base;
    int* dJ = dI + npairs;
    double* dE = (double*)(((uintptr_t)(dJ + npairs) + 15) & ~(uintptr_t)15);
    double* dD = dE + npairs;
    unsigned* dV = (unsigned*)(dD + npairs);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(dI, I, sizeof(int) * npairs, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess) return cudaFail(e, "copy pairs");
    if ((e = cudaMemcpyAsync(dJ, J, sizeof(int) * npairs, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess) return cudaFail(e, "copy pairs");
    if ((e = launchPairBatch(c->d, c->tables, npairs, dI, dJ, dE, dV, dD, c->stream)) != cudaSuccess) return cudaFail(e, "pair kernel");
    if ((e = cudaMemcpyAsync(E, dE, sizeof(double) * npairs, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy energies");
    if (V && (e = cudaMemcpyAsync(V, dV, sizeof(unsigned) * npairs, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy verdicts");
    if (D && (e = cudaMemcpyAsync(D, dD, sizeof(double) * npairs, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy distances");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "pair energies");
    return SC_OK;
}

int sc_pair_energy(sc_context* ctx, int i, int j, double* e) {
    if (!e) return fail(SC_ERR_ARG, "null argument");
    return sc_pair_energies(ctx, 1, &i, &j, e, nullptr, nullptr);
}

static int oneToAllImpl(Context* c, int ntargets, const int* targets, const TrialSlot* trialDev, double* out) {
    int rc;
    if ((rc = c->scratch((size_t)ntargets * (sizeof(int) + sizeof(double)) + 64))) return rc;
    int* dT = (int*)c->dScratch;
    double* dO = (double*)(((uintptr_t)(dT + ntargets) + 15) & ~(uintptr_t)15);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(dT, targets, sizeof(int) * ntargets, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess) return cudaFail(e, "copy targets");
    if ((e = launchOneToAll(c->d, c->tables, ntargets, dT, trialDev, dO, c->stream)) != cudaSuccess) return cudaFail(e, "one-to-all kernel");
    if ((e = cudaMemcpyAsync(out, dO, sizeof(double) * ntargets, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy energies");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "one-to-all");
    return SC_OK;
}

int sc_one_to_all(sc_context* ctx, int ntargets, const int* targets, double* out) {
    if (!ctx || ntargets < 0 || (ntargets > 0 && (!targets || !out))) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    int n = (int)c->conf.p.size();
    for (int k = 0; k < ntargets; ++k) if (targets[k] < 0 || targets[k] >= n) return fail(SC_ERR_ARG, "target out of range");
    if (ntargets == 0) return SC_OK;
    int rc = c->ensureDevice();
    if (rc) return rc;
    return oneToAllImpl(c, ntargets, targets, nullptr, out);
}

int sc_all_to_all(sc_context* ctx, double* out) {
    if (!ctx || !out) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    int rc = c->ensureDevice();
    if (rc) return rc;
    cudaError_t e;
    if ((e = launchAllToAll(c->d, c->tables, nullptr, c->dPartial, c->nPartial, c->dScalars, c->stream)) != cudaSuccess) return cudaFail(e, "all-to-all kernel");
    if ((e = cudaMemcpyAsync(out, c->dScalars, sizeof(double), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy energy");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "all-to-all");
    return SC_OK;
}

int sc_alignment_order(sc_context* ctx, double* out) {
    if (!ctx || !out) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    int rc = c->ensureDevice();
    if (rc) return rc;
    if (c->hostNewer && (rc = c->uploadState())) return rc;
    cudaError_t e;
    if ((e = launchAlignment(c->d, c->dPartial, c->nPartial, c->dScalars, c->stream)) != cudaSuccess) return cudaFail(e, "alignment kernel");
    if ((e = cudaMemcpyAsync(out, c->dScalars, sizeof(double), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "alignment");
    return SC_OK;
}

// Largest eigenvalue and its unit eigenvector of a symmetric 3x3 matrix (cyclic Jacobi).
static void largestEigen(double a[3][3], double* value, double vec[3]) {
    double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        if (off < 1e-30) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (a[p][q] == 0.0) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {      // a = J^T a J
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int best = 0;
    for (int k = 1; k < 3; ++k) if (a[k][k] > a[best][best]) best = k;
    *value = a[best][best];
    for (int k = 0; k < 3; ++k) vec[k] = v[k][best];
}

int sc_nematic_order(sc_context* ctx, double* s2, double director[3]) {
    if (!ctx || !s2) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    int rc = c->ensureDevice();
    if (rc) return rc;
    cudaError_t e;
    if ((e = launchAxisMoments(c->d, c->tables, c->dScalars, c->stream)) != cudaSuccess) return cudaFail(e, "axis moments");
    double m[7];
    if ((e = cudaMemcpyAsync(m, c->dScalars, sizeof m, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "nematic order");
    if (m[0] < 1.0) {
        *s2 = 0.0;
        if (director) director[0] = director[1] = director[2] = 0.0;
        return SC_OK;
    }
    const double n = m[0];
    double q[3][3] = {{1.5 * m[1] / n - 0.5, 1.5 * m[4] / n, 1.5 * m[5] / n},
                      {1.5 * m[4] / n, 1.5 * m[2] / n - 0.5, 1.5 * m[6] / n},
                      {1.5 * m[5] / n, 1.5 * m[6] / n, 1.5 * m[3] / n - 0.5}};
    double d[3];
    largestEigen(q, s2, d);
    if (director) for (int k = 0; k < 3; ++k) director[k] = d[k];
    return SC_OK;
}

int sc_mol_to_others(sc_context* ctx, int first, int size, double* out) {
    if (!ctx || !out) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    if (first < 0 || size <= 0 || first + size > (int)c->conf.p.size()) return fail(SC_ERR_ARG, "molecule range out of bounds");
    int rc = c->ensureDevice();
    if (rc) return rc;
    cudaError_t e;
    if ((e = launchMolToOthers(c->d, c->tables, first, size, c->dScalars, c->stream)) != cudaSuccess) return cudaFail(e, "mol2others kernel");
    if ((e = cudaMemcpyAsync(out, c->dScalars, sizeof(double), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy energy");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "mol2others");
    return SC_OK;
}

static void rotateParticle(Particle& p, int g, double angle, const double* ax, int positive) {
    // Particle::pscRotate (scOOP/structures/particle.h:182-272) with the sign given
    double vc = cos(angle);
    double vs = positive ? sqrt(1.0 - vc * vc) : -sqrt(1.0 - vc * vc);
    double qw = vc, qx = ax[0] * vs, qy = ax[1] * vs, qz = ax[2] * vs;
    double t2 = qw * qx, t3 = qw * qy, t4 = qw * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
           t9 = qy * qz, t10 = -qz * qz;
    double d1 = t8 + t10, d2 = t6 - t4, d3 = t3 + t7, d4 = t4 + t6, d5 = t5 + t10, d6 = t9 - t2, d7 = t7 - t3,
           d8 = t2 + t9, d9 = t5 + t8;
    auto rot = [&](Vec3& v) {
        double nx = 2.0 * (d1 * v.x + d2 * v.y + d3 * v.z) + v.x;
        double ny = 2.0 * (d4 * v.x + d5 * v.y + d6 * v.z) + v.y;
        double nz = 2.0 * (d7 * v.x + d8 * v.y + d9 * v.z) + v.z;
        v = {nx, ny, nz};
    };
    rot(p.dir);
    if (g != SCN && g != SCA) {
        int m = isTwoPatch(g) ? 2 : 1;
        for (int k = 0; k < m; ++k) { rot(p.pd[k]); rot(p.ps[2 * k]); rot(p.ps[2 * k + 1]); }
    }
    if (isChiral(g)) {
        int m = (g == TCHPSC || g == TCHCPSC) ? 2 : 1;
        for (int k = 0; k < m; ++k) rot(p.ch[k]);
    }
    // partRotate: patchdir[0].ortogonalise(dir) (movecreator.cpp:1007)
    double dp = p.pd[0].x * p.dir.x + p.pd[0].y * p.dir.y + p.pd[0].z * p.dir.z;
    p.pd[0].x -= dp * p.dir.x; p.pd[0].y -= dp * p.dir.y; p.pd[0].z -= dp * p.dir.z;
}

static int trialImpl(Context* c, int target, const Particle& trial, double* eOld, double* eNew) {
    TrialSlot ts;
    ts.pos = make_double4_32a(trial.pos.x, trial.pos.y, trial.pos.z, (double)c->compactOf[trial.type]);
    ts.dir = make_double4_32a(trial.dir.x, trial.dir.y, trial.dir.z, 0.0);
    for (int k = 0; k < 2; ++k) { ts.patch.pd[k][0] = trial.pd[k].x; ts.patch.pd[k][1] = trial.pd[k].y; ts.patch.pd[k][2] = trial.pd[k].z; }
    for (int k = 0; k < 4; ++k) { ts.patch.ps[k][0] = trial.ps[k].x; ts.patch.ps[k][1] = trial.ps[k].y; ts.patch.ps[k][2] = trial.ps[k].z; }
    for (int k = 0; k < 2; ++k) { ts.patch.ch[k][0] = trial.ch[k].x; ts.patch.ch[k][1] = trial.ch[k].y; ts.patch.ch[k][2] = trial.ch[k].z; }
    cudaError_t e;
    if ((e = cudaMemcpyAsync(c->dTrial, &ts, sizeof ts, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess) return cudaFail(e, "copy trial");
    int rc;
    double v;
    if ((rc = oneToAllImpl(c, 1, &target, nullptr, &v))) return rc;
    *eOld = v;
    if ((rc = oneToAllImpl(c, 1, &target, c->dTrial, &v))) return rc;
    *eNew = v;
    c->trialTarget = target;
    c->trialState = trial;
    return SC_OK;
}

int sc_trial_displace(sc_context* ctx, int target, const double dr[3], double* eOld, double* eNew) {
    if (!ctx || !dr || !eOld || !eNew) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    if (target < 0 || target >= (int)c->conf.p.size()) return fail(SC_ERR_ARG, "target out of range");
    int rc = c->downloadState();
    if (rc) return rc;
    if ((rc = c->ensureDevice())) return rc;
    Particle t = c->conf.p[target];
    t.pos.x += dr[0]; t.pos.y += dr[1]; t.pos.z += dr[2];
    return trialImpl(c, target, t, eOld, eNew);
}

int sc_trial_rotate(sc_context* ctx, int target, double angle, const double axis[3], int positive, double* eOld,
                    double* eNew, sc_particle* state) {
    if (!ctx || !axis || !eOld || !eNew) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    if (target < 0 || target >= (int)c->conf.p.size()) return fail(SC_ERR_ARG, "target out of range");
    int rc = c->downloadState();
    if (rc) return rc;
    if ((rc = c->ensureDevice())) return rc;
    Particle t = c->conf.p[target];
    rotateParticle(t, c->topo.ia[t.type][t.type].geotype[0], angle, axis, positive);
    if (state) toParticle(t, state);
    return trialImpl(c, target, t, eOld, eNew);
}

int sc_accept_trial(sc_context* ctx) {
    if (!ctx) return fail(SC_ERR_ARG, "null context");
    Context* c = C(ctx);
    if (c->trialTarget < 0) return fail(SC_ERR_STATE, "no trial move pending");
    int rc = c->downloadState();
    if (rc) return rc;
    c->conf.p[c->trialTarget] = c->trialState;
    c->trialTarget = -1;
    c->hostNewer = true;
    return SC_OK;
}

int sc_trial_volume(sc_context* ctx, double psch, double* eNew) {
    if (!ctx || !eNew) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    DeviceScope dev(c->device);
    int rc = c->ensureDevice();
    if (rc) return rc;
    if ((rc = c->downloadState())) return rc;
    double box[3] = {c->conf.box.x + psch, c->conf.box.y + psch, c->conf.box.z + psch};
    if (!(box[0] > 0 && box[1] > 0 && box[2] > 0)) return fail(SC_ERR_ARG, "box edge would not be positive");
    cudaError_t e;
    double* dBox = c->dScalars + 8;
    if ((e = cudaMemcpyAsync(dBox, box, sizeof box, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess) return cudaFail(e, "copy box");
    if ((e = launchAllToAll(c->d, c->tables, dBox, c->dPartial, c->nPartial, c->dScalars, c->stream)) != cudaSuccess) return cudaFail(e, "all-to-all kernel");
    if ((e = cudaMemcpyAsync(eNew, c->dScalars, sizeof(double), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) return cudaFail(e, "copy energy");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cudaFail(e, "volume trial");
    return SC_OK;
}

int sc_default_run(const sc_context* ctx, sc_run_params* p) {
    if (!ctx || !p) return fail(SC_ERR_ARG, "null argument");
    const Options& o = C(ctx)->opts;
    std::memset(p, 0, sizeof *p);
    p->nsweeps = o.nsweeps;
    p->seed = (unsigned long long)o.seed;
    p->temper = o.temper;
    p->press = o.press;
    p->ptype = o.ptype;
    // shave volume moves per sweep on average (updater.cpp:90), whatever the coupling type
    p->volume_every = (o.shave > 0) ? (int)(1.0 / o.shave + 0.5) : 0;
    if (p->volume_every < 1 && o.shave > 0) p->volume_every = 1;
    p->transmx = o.transmx;
    p->rot_angle = o.rot_angle;
    p->edge_mx = o.edge_mx;
    p->chainprob = o.chainprob;
    p->chainmmx = o.chainmmx;
    p->chain_angle = o.chain_angle;
    p->check_every = 100;
    p->variant = -1;       // sc_tune's choice for this context, else the dataflow sweep
    p->grand_every = (int)o.nGrandCanon;
    // no switchable particle: no switch moves (initSwitchList, inicializer.cpp:77-81)
    p->switchprob = C(ctx)->anySwitch ? o.switchprob : 0.0;
    return SC_OK;
}

int sc_grand_species(const sc_context* ctx, int* count) {
    if (!ctx || !count) return fail(SC_ERR_ARG, "null argument");
    *count = (int)C(ctx)->grand.size();
    return SC_OK;
}

int sc_write_top_last(sc_context* ctx, const char* path) {
    if (!ctx || !path) return fail(SC_ERR_ARG, "null argument");
    const Context* c = C(ctx);
    std::string out;
    size_t pos = 0;
    bool seen = false;
    while (pos < c->topText.size() && !seen) {
        size_t e = c->topText.find('\n', pos);
        std::string line = c->topText.substr(pos, e == std::string::npos ? std::string::npos : e - pos + 1);
        pos = e == std::string::npos ? c->topText.size() : e + 1;
        out += line;
        if (line.compare(0, 8, "[System]") == 0) seen = true;
    }
    if (!seen) return fail(SC_ERR_STATE, "Error writing Topology [System] not found");
    if (!out.empty() && out.back() != '\n') out += '\n';
    for (int m = 0; m < c->conf.molTypeCount; ++m) {
        const int size = std::max(1, (int)c->topo.mols[m].types.size());
        char buf[256];
        std::snprintf(buf, sizeof buf, "%s %d\n", c->topo.mols[m].name.c_str(),
                      (c->conf.first[m + 1] - c->conf.first[m]) / size);
        out += buf;
    }
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(SC_ERR_IO, std::string("cannot write ") + path);
    std::fwrite(out.data(), 1, out.size(), f);
    std::fclose(f);
    return SC_OK;
}

int sc_grand_stats_get(const sc_context* ctx, int k, sc_grand_stats* out) {
    if (!ctx || !out) return fail(SC_ERR_ARG, "null argument");
    const Context* c = C(ctx);
    if (k < 0 || k >= (int)c->grand.size()) return fail(SC_ERR_ARG, "grand-canonical species index out of range");
    const Context::Grand& g = c->grand[k];
    std::memset(out, 0, sizeof *out);
    out->mol_type = g.molType;
    out->type = g.type;
    out->count = c->conf.first[g.molType + 1] - c->conf.first[g.molType];
    out->activity = g.activity;
    out->chem_pot = g.chemPot;
    out->steps = g.steps;
    out->ins_acc = g.insAcc; out->ins_rej = g.insRej;
    out->del_acc = g.delAcc; out->del_rej = g.delRej;
    out->average_particles = g.steps > 0 ? g.countSum / (double)g.steps : 0.0;
    return SC_OK;
}

int sc_simulate(sc_context* ctx, const sc_run_params* p, sc_run_stats* stats) {
    if (!ctx || !p || !stats) return fail(SC_ERR_ARG, "null argument");
    DeviceScope dev(C(ctx)->device);
    return runSweeps(C(ctx), *p, *stats);
}

int sc_screen_survivors(sc_context* ctx, int ntargets, const int* targets, long cap, int* i, int* j,
                        unsigned char* stage_b, long* count) {
    if (!ctx || !count || cap < 0 || (cap > 0 && (!i || !j || !stage_b))) return fail(SC_ERR_ARG, "null argument");
    DeviceScope dev(C(ctx)->device);
    return screenSurvivors(C(ctx), targets ? ntargets : (int)C(ctx)->conf.p.size(), targets, cap, i, j, stage_b, count);
}

int sc_get_step_sizes(sc_context* ctx, sc_step_sizes* out) {
    if (!ctx || !out) return fail(SC_ERR_ARG, "null argument");
    Context* c = C(ctx);
    initStepSizes(c);
    std::memset(out, 0, sizeof *out);
    for (int t = 0; t < MAXT && t < 40; ++t) {
        out->trans[t] = c->trans[t].mx; out->rot_cos[t] = c->rot[t].mx;
        out->acc_trans[t] = c->trans[t].acc; out->rej_trans[t] = c->trans[t].rej;
        out->acc_rot[t] = c->rot[t].acc; out->rej_rot[t] = c->rot[t].rej;
    }
    for (int m = 0; m < Context::kMaxChainSteps && m < 8; ++m) {
        out->chain_trans[m] = c->chainm[m].mx; out->chain_rot_cos[m] = c->chainr[m].mx;
        out->acc_chain_trans[m] = c->chainm[m].acc; out->rej_chain_trans[m] = c->chainm[m].rej;
        out->acc_chain_rot[m] = c->chainr[m].acc; out->rej_chain_rot[m] = c->chainr[m].rej;
    }
    out->edge = c->edge.mx;
    out->acc_edge = c->edge.acc;
    out->rej_edge = c->edge.rej;
    out->adjustments = c->adjustments;
    return SC_OK;
}

int sc_adjust_steps(sc_context* ctx) {
    if (!ctx) return fail(SC_ERR_ARG, "null context");
    return adjustSteps(C(ctx));
}

int sc_equilibrate(sc_context* ctx, const sc_run_params* p, long nequil, long adjust, sc_run_stats* stats) {
    if (!ctx || !p || !stats) return fail(SC_ERR_ARG, "null argument");
    DeviceScope dev(C(ctx)->device);
    return equilibrate(C(ctx), *p, nequil, adjust, *stats);
}

int sc_tune(sc_context* ctx, const sc_run_params* p, int sweeps, sc_run_params* best, double* rates, int* ncand) {
    if (!ctx || !p || !best) return fail(SC_ERR_ARG, "null argument");
    DeviceScope dev(C(ctx)->device);
    return tuneSweeps(C(ctx), *p, sweeps, *best, rates, ncand);
}

struct sc_replicas {
    void* impl;
};

int sc_replicas_create(sc_context* const* systems, int nrep, const double* temperatures, const int* ladder,
                       sc_replicas** out) {
    if (!systems || !temperatures || !out || nrep < 1) return fail(SC_ERR_ARG, "null argument");
    std::vector<Context*> sys(nrep);
    for (int k = 0; k < nrep; ++k) sys[k] = systems[k];
    if (ladder)
        for (int k = 0; k < nrep; ++k)
            if (ladder[k] < 0 || ladder[k] >= nrep) return fail(SC_ERR_ARG, "ladder id out of range");
    void* impl = nullptr;
    int rc = createReplicas(sys.data(), nrep, temperatures, ladder, &impl);
    if (rc) return rc;
    *out = new sc_replicas{impl};
    return SC_OK;
}

int sc_replicas_run(sc_replicas* r, const sc_run_params* p, int exchange_every, sc_run_stats* stats,
                    double* temperatures, double* energies, long* tried, long* accepted) {
    if (!r || !p || !stats) return fail(SC_ERR_ARG, "null argument");
    if (exchange_every < 0) return fail(SC_ERR_ARG, "exchange_every must be >= 0");
    return runReplicas(r->impl, *p, exchange_every, *stats, temperatures, energies, tried, accepted);
}

int sc_replicas_destroy(sc_replicas* r) {
    if (!r) return fail(SC_ERR_ARG, "null argument");
    destroyReplicas(r->impl);
    delete r;
    return SC_OK;
}

}  // extern "C"
