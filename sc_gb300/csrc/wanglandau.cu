// wanglandau.cu -- Wang-Landau weights and histogram: the reference's wl.dat input and
// output (WangLandau::initCalc / write / endWangLandau, scOOP/mc/wanglandau.cpp:139-299,
// 404-433), the starting order parameters (WangLandau::init, :49-137) and the device record
// the move kernels bias with (sweep.cu: wlProposal, kWlCells, kVolumeAccept, kWlEndSweep).

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sc_gb300.h"
#include "sc_context.h"
#include "wanglandau.h"

namespace scg {

bool readFile(const char* path, std::string& out);   // sc_context.cu

// Weights and histogram of one run, shared by its walkers (sc_wl_share).
struct WlTableHost {
    WlTable h{};                     // host values; h.base / h.hist / h.hist0 are device arrays
    std::vector<double> base;        // host copies of the arrays
    std::vector<long long> hist, hist0;
    WlTable* d = nullptr;            // the device record
    int device = -1;
    bool onDevice = false;           // the device copy is the current one
    ~WlTableHost() {
        if (!d) return;
        DeviceScope dev(device);
        cudaFree(d);
        cudaFree(h.base);
        cudaFree(h.hist);
        cudaFree(h.hist0);
    }
};

struct WlHost {
    WlDev h{};                       // host values of the walker record (h.tab: device table)
    std::shared_ptr<WlTableHost> T;  // its table
    WlDev* d = nullptr;              // the device record
    int device = -1;
    bool onDevice = false;
};

// Bins of the current configuration (WangLandau::init): order 1 needs the system centre
// (Conf::massCenter, scOOP/structures/Conf.cpp:78-95, over anInt-wrapped positions,
// weighted by the Ia_param volumes; sysvolume as Inicializer sums it, inicializer.cpp:32-34);
// order 7 counts the particles 1..N-1 of type wlmtype in contact with particle 0
// (contParticlesAll, wanglandau.h:603-615).
static int wlOrders(const Context* c, WlDev& w, std::string& err) {
    const std::vector<Particle>& p = c->conf.p;
    const int n = (int)p.size();
    double sv = 0.0, cm[3] = {0, 0, 0}, k[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) sv += c->topo.ia[p[i].type][p[i].type].volume;
    for (int i = 0; i < n; ++i) {
        const double v = c->topo.ia[p[i].type][p[i].type].volume;
        const double r[3] = {p[i].pos.x, p[i].pos.y, p[i].pos.z};
        for (int d = 0; d < 3; ++d) {
            cm[d] += (r[d] - anInt(r[d])) * v;
            k[d] += v * anInt(r[d]);
        }
    }
    w.sysvol = sv;
    for (int d = 0; d < 3; ++d) {
        w.syscm[d] = cm[d] / sv;
        w.cmK[d] = k[d];
    }
    const double box[3] = {c->conf.box.x, c->conf.box.y, c->conf.box.z};
    for (int q = 0; q < 2; ++q) w.cur[q] = 0;
    for (int q = 0; q < w.dim; ++q) {
        switch (w.wlm[q]) {
        case 1: w.cur[q] = wlZOrder(w, q, p[0].pos.z, w.syscm[2], box[2]); break;
        case 3: w.cur[q] = wlOrientOrder(w, q, p[0].dir.z); break;
        case 4: {
            const double p0[3] = {p[0].pos.x, p[0].pos.y, p[0].pos.z}, p1[3] = {p[1].pos.x, p[1].pos.y, p[1].pos.z};
            w.cur[q] = wlDistOrder(w, q, p0, p1, box);
            break;
        }
        case 7: {
            long long cnt = 0;
            const double p0[3] = {p[0].pos.x, p[0].pos.y, p[0].pos.z};
            for (int i = 1; i < n; ++i) {
                const double pi[3] = {p[i].pos.x, p[i].pos.y, p[i].pos.z};
                if (p[i].type == c->opts.wlmtype && wlInContact(pi, p0, box)) ++cnt;
            }
            w.contacts = cnt;
            w.cur[q] = wlContactOrder(w, q, cnt);
            break;
        }
        case 8: w.cur[q] = wlBoxOrder(w, q, box[0]); break;
        case 9: w.cur[q] = wlBoxOrder(w, q, box[1]); break;
        default: break;
        }
        if (w.cur[q] < 0 || w.cur[q] >= w.len[q]) {
            char b[200];
            snprintf(b, sizeof b, "Wang-Landau: starting order parameter %g out of range (%g - %g)",
                     w.dorder[q] * (double)w.cur[q] + w.minorder[q], w.minorder[q],
                     w.minorder[q] + w.dorder[q] * w.len[q]);
            err = b;
            return SC_ERR_RANGE;
        }
    }
    return SC_OK;
}

// WangLandau::initCalc: '#' starts a comment, blank lines are skipped; the first line holds
// alpha, then one line per bin: "order weight hist" (one order parameter) or "order0
// order1 weight hist" (two, order0 running fastest).  The bin widths follow from the first
// and the last line.
static int wlParse(const std::string& text, WlHost& W, std::string& err) {
    std::istringstream in(text);
    std::string line;
    int i = 0, fields = 0;
    double f[4] = {0, 0, 0, 0};
    WlDev& w = W.h;
    WlTableHost& T = *W.T;
    w.len[0] = 0;
    w.len[1] = 0;
    T.base.clear();
    T.hist.clear();
    while (std::getline(in, line)) {
        size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        size_t a = line.find_first_not_of(" \t\r\n"), b = line.find_last_not_of(" \t\r\n");
        if (a == std::string::npos) continue;
        line = line.substr(a, b - a + 1);
        if (i == 0) {
            if (sscanf(line.c_str(), "%le", &T.h.alpha) != 1) { err = "Wang-Landau file: could not read alpha at the beginning"; return SC_ERR_PARSE; }
            ++i;
            continue;
        }
        fields = sscanf(line.c_str(), "%le %le %le %le", &f[0], &f[1], &f[2], &f[3]);
        if (fields == 3) {
            if (i == 1) w.minorder[0] = f[0];
            T.base.push_back(f[1]);
            T.hist.push_back((long long)f[2]);
            w.len[0]++;
        } else if (fields == 4) {
            if (i == 1) { w.minorder[0] = f[0]; w.minorder[1] = f[1]; }
            if (w.minorder[1] == f[1]) w.len[0]++;
            T.base.push_back(f[2]);
            T.hist.push_back((long long)f[3]);
        } else {
            err = "Wang-Landau file: could not read the order parameter at line " + std::to_string(i);
            return SC_ERR_PARSE;
        }
        ++i;
    }
    const long total = (long)T.base.size();
    if (total < 2 || w.len[0] < 2) { err = "Wang-Landau file: fewer than two bins"; return SC_ERR_PARSE; }
    if (fields == 4) {
        w.len[1] = (int)(total / w.len[0]);
        if (w.len[1] < 2 || (long)w.len[0] * w.len[1] != total) {
            err = "Wang-Landau file: the bin lines do not form a grid";
            return SC_ERR_PARSE;
        }
        w.dorder[1] = (f[1] - w.minorder[1]) / (w.len[1] - 1);
        w.dim = 2;
    } else {
        if (w.len[0] != total) { err = "Wang-Landau file: lines of two kinds"; return SC_ERR_PARSE; }
        w.len[1] = 1;
        w.dorder[1] = 0.0;
        w.minorder[1] = 0.0;
        w.dim = 1;
    }
    w.dorder[0] = (f[0] - w.minorder[0]) / (w.len[0] - 1);
    // WangLandau::init: a negligible alpha samples with fixed weights
    if (T.h.alpha < kWlAlphaTol / 100) T.h.alpha = 0.0;
    T.hist0 = T.hist;
    return SC_OK;
}

bool wlActive(const Context* c) { return c->wl && c->opts.wlm[0] > 0; }

WlDev* wlDevice(const Context* c) { return wlActive(c) && c->wl->onDevice ? c->wl->d : nullptr; }

int wlCheckRun(const Context* c, const sc_run_params& p) {
    if (c->opts.wlm[0] > 0 && !c->wl)
        return fail(SC_ERR_STATE, "options wlm > 0: the Wang-Landau weights must be loaded first (sc_wl_load; the "
                                  "reference reads wl.dat)");
    if (!wlActive(c)) return SC_OK;
    if (p.delayed) return fail(SC_ERR_UNSUPPORTED, "Wang-Landau weights with delayed acceptance");
    if (p.chainprob > 0) {
        for (int q = 0; q < 2; ++q) {
            const int i = c->wl->h.part[q];
            if (i >= 0 && c->molInfo[i].z > 1)
                return fail(SC_ERR_UNSUPPORTED, "Wang-Landau: a particle of the order parameters belongs to a chain "
                                                "and chain moves are on");
        }
        // order 7: chain moves of chains holding counted particles would change the count
        // outside the serialised cells
        if (c->wl->h.useContacts) {
            for (size_t i = 0; i < c->conf.p.size(); ++i)
                if (c->conf.p[i].type == c->opts.wlmtype && c->molInfo[i].z > 1)
                    return fail(SC_ERR_UNSUPPORTED, "Wang-Landau order 7: particles of type wlmtype belong to chains "
                                                    "and chain moves are on");
        }
    }
    return SC_OK;
}

// The table on the device (allocated on first use; arrays copied when `arrays`).
static int tableUpload(WlTableHost& T, int device, bool arrays) {
    const size_t nb = T.base.size();
    cudaError_t r;
    DeviceScope dev(device);
    if (!T.d) {
        if ((r = cudaMalloc((void**)&T.d, sizeof(WlTable))) != cudaSuccess) return cudaFail(r, "cudaMalloc (Wang-Landau)");
        if ((r = cudaMalloc((void**)&T.h.base, sizeof(double) * nb)) != cudaSuccess) return cudaFail(r, "cudaMalloc (Wang-Landau)");
        if ((r = cudaMalloc((void**)&T.h.hist, sizeof(long long) * nb)) != cudaSuccess) return cudaFail(r, "cudaMalloc (Wang-Landau)");
        if ((r = cudaMalloc((void**)&T.h.hist0, sizeof(long long) * nb)) != cudaSuccess) return cudaFail(r, "cudaMalloc (Wang-Landau)");
        T.device = device;
        arrays = true;
    }
    if (arrays) {
        cudaMemcpy(T.h.base, T.base.data(), sizeof(double) * nb, cudaMemcpyHostToDevice);
        cudaMemcpy(T.h.hist, T.hist.data(), sizeof(long long) * nb, cudaMemcpyHostToDevice);
        cudaMemcpy(T.h.hist0, T.hist0.data(), sizeof(long long) * nb, cudaMemcpyHostToDevice);
    }
    if ((r = cudaMemcpy(T.d, &T.h, sizeof(WlTable), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cudaFail(r, "upload Wang-Landau table");
    T.onDevice = true;
    return SC_OK;
}

// The device copies back to the host: the walker's record and its table (every walker of a
// shared table may have moved: the whole device is synchronised).
static int wlDownload(Context* c) {
    WlHost& W = *c->wl;
    WlTableHost& T = *W.T;
    cudaError_t r;
    DeviceScope dev(c->device);
    if (W.onDevice) {
        cudaSetDevice(W.device);
        cudaDeviceSynchronize();
        if ((r = cudaMemcpy(&W.h, W.d, sizeof(WlDev), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cudaFail(r, "download Wang-Landau record");
    }
    if (T.onDevice) {
        cudaSetDevice(T.device);
        cudaDeviceSynchronize();
        if ((r = cudaMemcpy(&T.h, T.d, sizeof(WlTable), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cudaFail(r, "download Wang-Landau table");
        const size_t nb = T.base.size();
        cudaMemcpy(T.base.data(), T.h.base, sizeof(double) * nb, cudaMemcpyDeviceToHost);
        cudaMemcpy(T.hist.data(), T.h.hist, sizeof(long long) * nb, cudaMemcpyDeviceToHost);
        cudaMemcpy(T.hist0.data(), T.h.hist0, sizeof(long long) * nb, cudaMemcpyDeviceToHost);
    }
    return SC_OK;
}

int wlPrepare(Context* c, bool hostChanged) {
    if (!wlActive(c)) return SC_OK;
    WlHost& W = *c->wl;
    WlTableHost& T = *W.T;
    std::string err;
    int rc;
    cudaError_t r;
    if (W.onDevice) {
        // the device record is the current one (bins, centre)
        if (c->stream) cudaStreamSynchronize(c->stream);
        if ((r = cudaMemcpy(&W.h, W.d, sizeof(WlDev), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cudaFail(r, "download Wang-Landau record");
        // the caller replaced the state: the bins and the centre follow it (the table stays)
        if (hostChanged && (rc = wlOrders(c, W.h, err))) return fail(rc, err);
    }
    if (T.onDevice && T.device != c->device)
        return fail(SC_ERR_UNSUPPORTED, "Wang-Landau walkers sharing weights must be on one device");
    if (!T.onDevice && (rc = tableUpload(T, c->device, true))) return rc;
    if (!W.d) {
        if ((r = cudaMalloc((void**)&W.d, sizeof(WlDev))) != cudaSuccess) return cudaFail(r, "cudaMalloc (Wang-Landau)");
        W.device = c->device;
    }
    W.h.chainSeen = 0;          // the run's counters start from zero
    W.h.cell[0] = W.h.cell[1] = -1;
    W.h.tab = T.d;
    if ((r = cudaMemcpy(W.d, &W.h, sizeof(WlDev), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cudaFail(r, "upload Wang-Landau record");
    W.onDevice = true;
    return SC_OK;
}

bool wlConverged(Context* c) {
    if (!wlActive(c) || !c->wl->T->onDevice) return false;
    int v = 0;
    cudaMemcpy(&v, &c->wl->T->d->converged, sizeof v, cudaMemcpyDeviceToHost);
    return v != 0;
}

void destroyWl(Context* c) {
    if (!c->wl) return;
    WlHost& W = *c->wl;
    if (W.d) {
        DeviceScope dev(W.device);
        cudaFree(W.d);
    }
    delete c->wl;       // the table goes with its last walker
    c->wl = nullptr;
}

static int wlLoad(Context* c, const std::string& text) {
    const int* m = c->opts.wlm;
    if (m[0] <= 0) return fail(SC_ERR_STATE, "options wlm is 0: no Wang-Landau order parameter to load weights for");
    for (int q = 0; q < 2; ++q) {
        if (m[q] == 0) continue;
        if (m[q] != 1 && m[q] != 3 && m[q] != 4 && m[q] != 7 && m[q] != 8 && m[q] != 9)
            return fail(SC_ERR_UNSUPPORTED, "Wang-Landau order parameter " + std::to_string(m[q]) +
                                                " (supported: 1, 3, 4, 7, 8, 9; the mesh-hole and pore orders 2, 5, 6 "
                                                "are not on the GPU path)");
    }
    if ((m[0] == 4 || m[1] == 4) && c->conf.p.size() < 2)
        return fail(SC_ERR_ARG, "Wang-Landau order 4 needs two particles");
    if (c->conf.p.empty()) return fail(SC_ERR_ARG, "no particles");
    int rc;
    if (c->devNewer && (rc = c->downloadState())) return rc;
    WlHost* W = new WlHost();
    W->T = std::make_shared<WlTableHost>();
    std::string err;
    if ((rc = wlParse(text, *W, err))) { delete W; return fail(rc, err); }
    WlDev& w = W->h;
    const int dimOpts = m[1] > 0 ? 2 : 1;
    if (w.dim != dimOpts) {
        delete W;
        return fail(SC_ERR_PARSE, "Wang-Landau file has " + std::to_string(w.dim) + " order parameter column(s), the "
                                  "options name " + std::to_string(dimOpts));
    }
    w.wlm[0] = m[0];
    w.wlm[1] = m[1];
    bool uses[10] = {};
    for (int q = 0; q < w.dim; ++q) uses[m[q]] = true;
    w.needCM = uses[1] ? 1 : 0;
    w.part[0] = (uses[1] || uses[3] || uses[4] || uses[7]) ? 0 : -1;
    w.part[1] = uses[4] ? 1 : -1;
    w.cell[0] = w.cell[1] = -1;
    w.useContacts = uses[7] ? 1 : 0;
    const int wt = c->opts.wlmtype;
    w.contactType = (wt >= 0 && wt < MAXT) ? c->compactOf[wt] : -1;
    for (int d = 0; d < 3; ++d) w.reach[d] = 0;
    w.contacts = 0;
    w.owner = 1;
    if ((rc = wlOrders(c, w, err))) { delete W; return fail(rc, err); }
    destroyWl(c);
    c->wl = W;
    return SC_OK;
}

static std::string wlFormat(const WlHost& W, const std::vector<double>& wt) {
    const WlDev& w = W.h;
    const WlTableHost& T = *W.T;
    std::string s;
    char b[128];
    snprintf(b, sizeof b, "%15.8e \n", T.h.alpha);
    s += b;
    if (w.dim == 1) {
        for (int i = 0; i < w.len[0]; ++i) {
            snprintf(b, sizeof b, "%15.8e %15.8e %ld \n", w.minorder[0] + i * w.dorder[0], wt[i], (long)T.hist[i]);
            s += b;
        }
    } else {
        for (int j = 0; j < w.len[1]; ++j) {
            for (int i = 0; i < w.len[0]; ++i) {
                const size_t k = (size_t)i + (size_t)w.len[0] * j;
                snprintf(b, sizeof b, "%15.8e %15.8e %15.8e %ld \n", w.minorder[0] + i * w.dorder[0],
                         w.minorder[1] + j * w.dorder[1], wt[k], (long)T.hist[k]);
                s += b;
            }
            s += " \n";
        }
    }
    return s;
}

static std::vector<double> wlWeights(const WlHost& W) {
    const WlTableHost& T = *W.T;
    std::vector<double> wt(T.base.size());
    for (size_t i = 0; i < wt.size(); ++i) wt[i] = T.base[i] - T.h.alpha * (double)(T.hist[i] - T.hist0[i]);
    return wt;
}

// Walkers 1..n-1 take walker 0's table: the reference's multiple walkers, which update one
// set of weights and one histogram (MPI shared windows, wanglandau.cpp:184-218); walker 0
// runs the flatness checks (update() on rank 0, wanglandau.h:66-120).
static int wlShare(Context* const* ws, int n) {
    if (n < 1) return fail(SC_ERR_ARG, "no walkers");
    for (int k = 0; k < n; ++k)
        if (!ws[k] || !wlActive(ws[k])) return fail(SC_ERR_STATE, "every walker needs Wang-Landau weights loaded");
    const WlDev& a = ws[0]->wl->h;
    for (int k = 1; k < n; ++k) {
        const WlDev& b = ws[k]->wl->h;
        bool same = a.dim == b.dim && a.len[0] == b.len[0] && a.len[1] == b.len[1];
        for (int q = 0; q < 2 && same; ++q)
            same = a.wlm[q] == b.wlm[q] && a.minorder[q] == b.minorder[q] && a.dorder[q] == b.dorder[q];
        if (!same) return fail(SC_ERR_ARG, "Wang-Landau walkers sharing weights need the same order parameters and bins");
        if (ws[k]->device != ws[0]->device) return fail(SC_ERR_ARG, "walkers sharing weights must be on one device");
    }
    for (int k = 1; k < n; ++k) {
        if (ws[k]->wl->T == ws[0]->wl->T) continue;
        ws[k]->wl->T = ws[0]->wl->T;
        ws[k]->wl->h.owner = 0;
    }
    ws[0]->wl->h.owner = 1;
    return SC_OK;
}

}  // namespace scg

using namespace scg;

struct sc_context : public Context {};

static int writeText(const char* path, const std::string& s) {
    FILE* f = fopen(path, "w");
    if (!f) return fail(SC_ERR_IO, std::string("cannot write ") + path);
    fwrite(s.data(), 1, s.size(), f);
    fclose(f);
    return SC_OK;
}

extern "C" {

int sc_wl_load_text(sc_context* ctx, const char* text) {
    if (!ctx || !text) return fail(SC_ERR_ARG, "null argument");
    return wlLoad(ctx, text);
}

int sc_wl_load(sc_context* ctx, const char* path) {
    if (!ctx || !path) return fail(SC_ERR_ARG, "null argument");
    std::string t;
    if (!readFile(path, t)) return fail(SC_ERR_IO, std::string("cannot read ") + path);
    return wlLoad(ctx, t);
}

int sc_wl_get_info(sc_context* ctx, sc_wl_info* out) {
    if (!ctx || !out) return fail(SC_ERR_ARG, "null argument");
    if (!ctx->wl) return fail(SC_ERR_STATE, "no Wang-Landau weights loaded");
    int rc = wlDownload(ctx);
    if (rc) return rc;
    const WlDev& w = ctx->wl->h;
    std::memset(out, 0, sizeof *out);
    out->dim = w.dim;
    for (int q = 0; q < 2; ++q) {
        out->wlm[q] = w.wlm[q];
        out->minorder[q] = w.minorder[q];
        out->dorder[q] = w.dorder[q];
        out->currorder[q] = (long)w.cur[q];
    }
    out->length[0] = w.len[0];
    out->length[1] = w.dim == 2 ? w.len[1] : 0;
    const WlTable& t = ctx->wl->T->h;
    out->alpha = t.alpha;
    out->updates = (long)t.updates;
    out->converged = t.converged;
    for (int d = 0; d < 3; ++d) out->syscm[d] = w.syscm[d];
    return SC_OK;
}

int sc_wl_share(sc_context* const* walkers, int n) {
    if (!walkers) return fail(SC_ERR_ARG, "null argument");
    std::vector<Context*> ws(n > 0 ? n : 0);
    for (int k = 0; k < n; ++k) ws[k] = walkers[k];
    return wlShare(ws.data(), n);
}

int sc_wl_get(sc_context* ctx, double* weights, long* hist) {
    if (!ctx) return fail(SC_ERR_ARG, "null context");
    if (!ctx->wl) return fail(SC_ERR_STATE, "no Wang-Landau weights loaded");
    int rc = wlDownload(ctx);
    if (rc) return rc;
    const WlHost& W = *ctx->wl;
    std::vector<double> wt = wlWeights(W);
    for (size_t i = 0; i < wt.size(); ++i) {
        if (weights) weights[i] = wt[i];
        if (hist) hist[i] = (long)W.T->hist[i];
    }
    return SC_OK;
}

int sc_wl_write(sc_context* ctx, const char* path) {
    if (!ctx || !path) return fail(SC_ERR_ARG, "null argument");
    if (!ctx->wl) return fail(SC_ERR_STATE, "no Wang-Landau weights loaded");
    int rc = wlDownload(ctx);
    if (rc) return rc;
    return writeText(path, wlFormat(*ctx->wl, wlWeights(*ctx->wl)));
}

int sc_wl_end(sc_context* ctx, const char* path) {
    if (!ctx || !path) return fail(SC_ERR_ARG, "null argument");
    if (!ctx->wl) return fail(SC_ERR_STATE, "no Wang-Landau weights loaded");
    int rc = wlDownload(ctx);
    if (rc) return rc;
    std::vector<double> wt = wlWeights(*ctx->wl);
    // WangLandau::endWangLandau shifts by the first bin's weight inside a loop over the
    // second dimension, which is empty for one order parameter: only 2-D weights move
    const WlDev& w = ctx->wl->h;
    if (w.dim == 2) {
        const double wmin = wt[0];
        for (double& x : wt) x -= wmin;
    }
    return writeText(path, wlFormat(*ctx->wl, wt));
}

}  // extern "C"
