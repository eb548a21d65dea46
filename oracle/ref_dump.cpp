// ref_dump.cpp -- golden-vector generator for the parity tests.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's own sources (scOOP/, read in place and never copied) into
// oracle/_ref/ref_dump.  It drives the reference's pair-energy routine on the
// three input files of a working directory and prints, as JSON on stdout, every
// number the parity tests compare against:
//
//   * derived interaction parameters      Topo::genParamPairs   scOOP/structures/topo.cpp:5-153
//   * particles after Conf::partVecInit   scOOP/structures/Conf.cpp:97-102, particle.cpp:3-79
//   * E(i,j) = PairE(i, j, conlist(i))    scOOP/mc/paire.h:1209-1220 for every ordered pair that
//     passes the sqmaxcut prefilter, with the branch verdicts re-derived from
//     the reference's own helpers (EPatch::closestDist, Psc::pscIntersect,
//     CPsc::cpscIntersect)
//   * oneToAllTrial(i) for every i        scOOP/mc/totalenergycalculator.h:383-415 (no pair list)
//   * allToAll                             scOOP/mc/totalenergycalculator.h:502-521
//   * scripted displacement / rotation trial moves with the resulting state and
//     dE, built from Vector::randomUnitSphere and Particle::pscRotate the way
//     MoveCreator::partDisplace / partRotate do (scOOP/mc/movecreator.cpp:947-1028)
//   * isotropic volume trials (ptype 1, scOOP/mc/movecreator.cpp:390-421)
//   * mol2othersTrial for each chain       scOOP/mc/totalenergycalculator.h:453-499
//
// Usage: ref_dump <workdir> [n_trials] [max_i]
//   workdir holds options, top.init, config.init; pairs are listed for i < max_i only.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <unistd.h>
#include <vector>

#include "mc/inicializer.h"
#include "mc/wanglandau.h"
#include "mc/paire.h"
#include "mc/randomGenerator.h"

MpiCout mcout(0);
Topo topo;
#ifdef RAN2
Ran2 ran2;
#else
Dsfmt ran2;
#endif

static FILE* out = stdout;

// JSON number, with Python's json tokens for non-finite values.
static const char* J(double v) {
    static char buf[16][40];
    static int k = 0;
    char* b = buf[k++ & 15];
    if (std::isnan(v)) snprintf(b, 40, "NaN");
    else if (std::isinf(v)) snprintf(b, 40, v > 0 ? "Infinity" : "-Infinity");
    else snprintf(b, 40, "%.17g", v);
    return b;
}

static void pv(const char* key, const Vector& v, bool comma = true) {
    fprintf(out, "\"%s\": [%s, %s, %s]%s", key, J(v.x), J(v.y), J(v.z), comma ? ", " : "");
}
static void parr(const char* key, const double* a, int n, bool comma = true) {
    fprintf(out, "\"%s\": [", key);
    for (int k = 0; k < n; ++k) fprintf(out, "%s%s", J(a[k]), k + 1 < n ? ", " : "");
    fprintf(out, "]%s", comma ? ", " : "");
}

static bool isPscF(int g) { return g == PSC || g == CHPSC || g == TPSC || g == TCHPSC; }
static bool isCpscF(int g) { return g == CPSC || g == CHCPSC || g == TCPSC || g == TCHCPSC; }

// Functor kinds in the order scOOP/mc/paire.cpp:29-77 assigns them (later rules override).
enum Kind { K_NONE = 0, K_SC_PSC_CPSC, K_SC_CPSC, K_SC_PSC, K_SC_SCN, K_SC_SCA,
            K_SP_WCA, K_SP_SPA, K_MIX_SCA_SPA, K_MIX_PSC_SP, K_MIX_CPSC_SP };

static int functorKind(int g, int o) {
    int k = K_NONE;
    if ((isCpscF(g) && isPscF(o)) || (isPscF(g) && isCpscF(o))) k = K_SC_PSC_CPSC;
    if (isCpscF(g) && isCpscF(o)) k = K_SC_CPSC;
    if (isPscF(g) && isPscF(o)) k = K_SC_PSC;
    if (g == SCN && o == SCN) k = K_SC_SCN;
    if (g == SCA && o == SCA) k = K_SC_SCA;
    if (g == SPN || o == SPN) k = K_SP_WCA;
    if (g == SPA && o == SPA) k = K_SP_SPA;
    if ((g == SCA && o == SPA) || (g == SPA && o == SCA)) k = K_MIX_SCA_SPA;
    if ((isPscF(g) && (o == SPA || o == SPN)) || ((g == SPA || g == SPN) && isPscF(o))) k = K_MIX_PSC_SP;
    if ((isCpscF(g) && (o == SPA || o == SPN)) || ((g == SPA || g == SPN) && isCpscF(o))) k = K_MIX_CPSC_SP;
    return k;
}

// Verdict bits; the oracle restatement and the CUDA kernels produce the same layout.
enum {
    V_EVAL = 1u << 0,   // passed the sqmaxcut prefilter (or the conlist is non-empty)
    V_WCA = 1u << 1,    // repulsive branch taken
    V_ATR = 1u << 2,    // attractive branch entered (cutoff / epsilon / exclusion tests passed)
    V_FAR = 1u << 3,    // MixSpSc isFar() true
    // SC-SC: bit 8+2c: first intersection test of patch combination c returned 2,
    //        bit 9+2c: second one returned 2 (c = pn1 + 2*pn2).
    // SC-sphere: bit 8+p: patch p has dist < rcut.
};

static Conf* gconf;

static void scGeo(int kind, const Ia_param& ia, bool& fCH, bool& sCH, bool& fT, bool& sT) {
    int g0 = ia.geotype[0], g1 = ia.geotype[1];
    fCH = sCH = fT = sT = false;
    if (kind == K_SC_PSC) {
        fCH = (g0 == CHPSC || g0 == TCHPSC); sCH = (g1 == CHPSC || g1 == TCHPSC);
        fT = (g0 == TPSC || g0 == TCHPSC);   sT = (g1 == TPSC || g1 == TCHPSC);
    } else if (kind == K_SC_CPSC) {
        fCH = (g0 == CHCPSC || g0 == TCHCPSC); sCH = (g1 == CHCPSC || g1 == TCHCPSC);
        fT = (g0 == TCPSC || g0 == TCHCPSC);   sT = (g1 == TCPSC || g1 == TCHCPSC);
    } else if (kind == K_SC_PSC_CPSC) {
        fCH = (g0 == CHPSC || g0 == CHCPSC || g0 == TCHPSC || g0 == TCHCPSC);
        sCH = (g1 == CHPSC || g1 == CHCPSC || g1 == TCHPSC || g1 == TCHCPSC);
        fT = (g0 == TCPSC || g0 == TCHCPSC || g0 == TPSC || g0 == TCHPSC);
        sT = (g1 == TCPSC || g1 == TCHCPSC || g1 == TPSC || g1 == TCHPSC);
    }
}

static unsigned verdict(Particle* p1, Particle* p2, ConList* con, double* distSqOut) {
    unsigned bits = 0;
    *distSqOut = -1.0;
    Vector r_cm = gconf->geo.image(&p1->pos, &p2->pos);
    double dotrcm = r_cm.dot(r_cm);
    if (dotrcm > topo.sqmaxcut && con->isEmpty) return 0;
    bits |= V_EVAL;
    const Ia_param& ia = topo.ia_params[p1->type][p2->type];
    int kind = functorKind(ia.geotype[0], ia.geotype[1]);
    double dist = sqrt(dotrcm);
    if (kind == K_SC_PSC || kind == K_SC_CPSC || kind == K_SC_PSC_CPSC || kind == K_SC_SCN || kind == K_SC_SCA) {
        Psc<WcaTruncSq> psc;
        CPsc<WcaTruncSq> cpsc;
        double distSq = psc.closestDist(r_cm, p1->dir, p2->dir, ia);
        *distSqOut = distSq;
        if (!(distSq > ia.rcutwcaSq)) bits |= V_WCA;
        if (!((distSq > ia.rcutSq) || ia.epsilon == 0.0 || ia.exclude)) {
            bits |= V_ATR;
            bool fCH, sCH, fT, sT;
            scGeo(kind, ia, fCH, sCH, fT, sT);
            for (int c = 0; c < 4; ++c) {
                int pn1 = c & 1, pn2 = c >> 1;
                if (pn1 && !fT) continue;
                if (pn2 && !sT) continue;
                Vector d1 = fCH ? p1->chdir[pn1] : p1->dir;
                Vector d2 = sCH ? p2->chdir[pn2] : p2->dir;
                Patch P1(p1->patchdir[pn1], p1->patchsides[2 * pn1], p1->patchsides[2 * pn1 + 1]);
                Patch P2(p2->patchdir[pn2], p2->patchsides[2 * pn2], p2->patchsides[2 * pn2 + 1]);
                Vector mr = -1.0 * r_cm;
                double T1, T2, S1, S2;
                bool firstPsc, secondPsc;
                if (kind == K_SC_PSC) { firstPsc = true; secondPsc = true; }
                else if (kind == K_SC_CPSC) { firstPsc = false; secondPsc = false; }
                else if (kind == K_SC_PSC_CPSC) {
                    int g0 = ia.geotype[0];
                    bool first = (g0 == PSC) || (g0 == CHPSC) || (g0 == TPSC) || (g0 == TCHPSC);
                    firstPsc = first; secondPsc = !first;
                } else continue;  // SCN / SCA: no intersections
                int a = firstPsc
                    ? psc.pscIntersect(d1, d2, P1, r_cm, T1, T2, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1])
                    : cpsc.cpscIntersect(d1, d2, P1, r_cm, T1, T2, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1]);
                if (a < 2) continue;
                bits |= 1u << (8 + 2 * c);
                int b = secondPsc
                    ? psc.pscIntersect(d2, d1, P2, mr, S1, S2, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0])
                    : cpsc.cpscIntersect(d2, d1, P2, mr, S1, S2, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0]);
                if (b >= 2) bits |= 1u << (9 + 2 * c);
            }
        }
    } else if (kind == K_MIX_SCA_SPA || kind == K_MIX_PSC_SP || kind == K_MIX_CPSC_SP) {
        // Point-to-segment distance as in the private MixSpSc::closestDist (paire.h:1077-1093).
        bool isp1Spc = (ia.geotype[0] < SP);
        const Particle* spc = isp1Spc ? p1 : p2;
        const Ia_param& iap = isp1Spc ? topo.ia_params[p1->type][p2->type] : topo.ia_params[p2->type][p1->type];
        Vector rc = isp1Spc ? r_cm : -1.0 * r_cm;
        auto cdist = [&](const Vector& d1, double& contt) {
            double halfl = iap.half_len[0];
            contt = DOT(d1, rc);
            double d = -halfl;
            if (contt >= halfl) d = halfl;
            else if (contt > -halfl) d = contt;
            Vector dv(-rc.x + d1.x * d, -rc.y + d1.y * d, -rc.z + d1.z * d);
            return DOT(dv, dv);
        };
        double contt;
        double distSq = cdist(spc->dir, contt);
        *distSqOut = distSq;
        bool isFar = (kind == K_MIX_CPSC_SP) && ((contt > iap.half_len[0]) || (contt < -iap.half_len[0]));
        if (isFar) bits |= V_FAR;
        if (distSq < iap.rcutwcaSq) bits |= V_WCA;
        if (!((distSq > iap.rcutSq) || iap.epsilon == 0.0 || iap.exclude || isFar)) {
            bits |= V_ATR;
            int g0 = iap.geotype[0];
            bool chiral = false, sec = false;
            if (kind == K_MIX_PSC_SP) { chiral = (g0 == CHPSC || g0 == TCHPSC); sec = (g0 == TPSC || g0 == TCHPSC); }
            if (kind == K_MIX_CPSC_SP) { chiral = (g0 == CHCPSC || g0 == TCHCPSC); sec = (g0 == TCPSC || g0 == TCHCPSC); }
            if (chiral) distSq = cdist(spc->chdir[0], contt);
            if (sqrt(distSq) < iap.rcut) bits |= 1u << 8;
            if (sec) {
                distSq = cdist(chiral ? spc->chdir[1] : spc->dir, contt);
                if (sqrt(distSq) < iap.rcut) bits |= 1u << 9;
            }
        }
    } else if (kind == K_SP_WCA) {
        *distSqOut = dotrcm;
        if (!(dist > ia.rcutwca)) bits |= V_WCA;
    } else if (kind == K_SP_SPA) {
        *distSqOut = dotrcm;
        if (!(dist > ia.rcut || ia.epsilon == 0.0 || ia.exclude)) {
            bits |= V_ATR;
            if (!(dist > ia.rcutwca)) bits |= V_WCA;
        }
    }
    return bits;
}

static double oneToAllFresh(PairE& pairE, int target) {
    ConList con = gconf->pvec.getConlist(target);
    double e = 0.0;
    for (int i = 0; i < target; ++i) e += pairE(&gconf->pvec[target], &gconf->pvec[i], &con);
    for (int i = target + 1; i < (int)gconf->pvec.size(); ++i) e += pairE(&gconf->pvec[target], &gconf->pvec[i], &con);
    return e;
}

static double allToAllFresh(PairE& pairE) {
    double e = 0.0;
    for (unsigned i = 1; i < gconf->pvec.size(); ++i) {
        ConList con = gconf->pvec.getConlist(i);
        for (unsigned j = 0; j < i; ++j) e += pairE(&gconf->pvec[i], &gconf->pvec[j], &con);
    }
    return e;
}

static void dumpParticle(const Particle& p, bool comma) {
    fprintf(out, "{");
    pv("pos", p.pos); pv("dir", p.dir);
    pv("pd0", p.patchdir[0]); pv("pd1", p.patchdir[1]);
    pv("ps0", p.patchsides[0]); pv("ps1", p.patchsides[1]); pv("ps2", p.patchsides[2]); pv("ps3", p.patchsides[3]);
    pv("ch0", p.chdir[0]); pv("ch1", p.chdir[1]);
    fprintf(out, "\"type\": %d, \"molType\": %d, \"switched\": %d}%s\n", p.type, p.molType, p.switched, comma ? "," : "");
}

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_dump <workdir> [n_trials]\n"); return 2; }
    if (chdir(argv[1]) != 0) { perror("chdir"); return 2; }
    int nTrials = argc > 2 ? atoi(argv[2]) : 64;
    int maxI = argc > 3 ? atoi(argv[3]) : 1 << 30;

    // Keep the reference's own progress prints off stdout (they go to stderr).
    fflush(stdout);
    int saved = dup(1);
    dup2(2, 1);

    FileNames files(0);
    Conf conf;
    gconf = &conf;
    Sim sim(&conf, &files, 0, 1);
    Inicializer init(&sim, &conf, &files);
    init.initTop();
    init.testChains();
    FILE* infile = fopen(files.configurationInFile, "r");
    if (!infile || !init.initConfig(&infile, conf.pvec)) { fprintf(stderr, "config read failed\n"); return 1; }
    fclose(infile);
    std::vector<Particle> beforeInit(conf.pvec.begin(), conf.pvec.end());
    conf.partVecInit();
    PairE pairE(&conf.geo);

    fflush(stdout);
    dup2(saved, 1);
    out = stdout;

    const int N = (int)conf.pvec.size();
    std::vector<int> used;
    for (int t = 0; t < MAXT; ++t) if (topo.ia_params[t][t].geotype[0] != 0) used.push_back(t);

    fprintf(out, "{\n");
    pv("box", conf.geo.box, false);
    fprintf(out, ",\n\"sqmaxcut\": %s, \"maxcut\": %s,\n", J(topo.sqmaxcut), J(topo.maxcut));
    fprintf(out, "\"options\": {\"temper\": %s, \"press\": %s, \"ptype\": %d, \"shave\": %s, \"chainprob\": %s, "
                 "\"transmx\": %s, \"rot_angle\": %s, \"edge_mx\": %s, \"chainmmx\": %s, \"chainr_angle\": %s, "
                 "\"nsweeps\": %ld, \"seed_pairlist\": %d},\n",
            J(sim.temper), J(sim.press), sim.ptype, J(sim.shave), J(sim.chainprob), J(sim.stat.trans[used[0]].mx), J(sim.stat.rot[used[0]].angle),
            J(sim.stat.edge.mx), J(sim.stat.chainm[0].mx), J(sim.stat.chainr[0].angle), sim.nsweeps, sim.pairlist_update);

    // Derived interaction parameters of every used type pair.
    fprintf(out, "\"ia_params\": [\n");
    for (size_t a = 0; a < used.size(); ++a) for (size_t b = 0; b < used.size(); ++b) {
        const Ia_param& p = topo.ia_params[used[a]][used[b]];
        fprintf(out, "{\"t1\": %d, \"t2\": %d, \"geotype\": [%d, %d], ", used[a], used[b], p.geotype[0], p.geotype[1]);
        fprintf(out, "\"sigma\": %s, \"epsilon\": %s, \"A\": %s, \"B\": %s, \"pdis\": %s, \"pswitch\": %s, "
                     "\"pswitchINV\": %s, \"rcut\": %s, \"rcutSq\": %s, \"rcutwca\": %s, \"rcutwcaSq\": %s, "
                     "\"volume\": %s, \"parallel\": %s, \"exclude\": %d, ",
                J(p.sigma), J(p.epsilon), J(p.A), J(p.B), J(p.pdis), J(p.pswitch), J(p.pswitchINV), J(p.rcut), J(p.rcutSq), J(p.rcutwca), J(p.rcutwcaSq),
                J(p.volume), J(p.parallel), (int)p.exclude);
        parr("pcangl", p.pcangl, 4); parr("pcanglsw", p.pcanglsw, 4); parr("pcoshalfi", p.pcoshalfi, 4);
        parr("psinhalfi", p.psinhalfi, 4); parr("csecpatchrot", p.csecpatchrot, 2); parr("ssecpatchrot", p.ssecpatchrot, 2);
        parr("len", p.len, 2); parr("half_len", p.half_len, 2); parr("chiral_cos", p.chiral_cos, 2);
        parr("chiral_sin", p.chiral_sin, 2, false);
        fprintf(out, "}%s\n", (a + 1 == used.size() && b + 1 == used.size()) ? "" : ",");
    }
    fprintf(out, "],\n");

    // Molecule parameters.
    fprintf(out, "\"molecules\": [\n");
    for (int m = 0; m < conf.pvec.molTypeCount; ++m) {
        MoleculeParams& mp = topo.moleculeParam[m];
        fprintf(out, "{\"size\": %d, \"first\": %d, \"count\": %d, \"bond1\": [%s, %s], \"bond2\": [%s, %s], "
                     "\"bondd\": [%s, %s], \"bondh\": [%s, %s], \"angle1\": [%s, %s], \"angle2\": [%s, %s]}%s\n",
                mp.molSize(), conf.pvec.first[m], conf.pvec.molCountOfType(m), J(mp.bond1c), J(mp.bond1eq), J(mp.bond2c), J(mp.bond2eq),
                J(mp.bonddc), J(mp.bonddeq), J(mp.bondhc), J(mp.bondheq), J(mp.angle1c), J(mp.angle1eq), J(mp.angle2c), J(mp.angle2eq),
                m + 1 < conf.pvec.molTypeCount ? "," : "");
    }
    fprintf(out, "],\n");

    fprintf(out, "\"particles_in\": [\n");
    for (int i = 0; i < N; ++i) dumpParticle(beforeInit[i], i + 1 < N);
    fprintf(out, "],\n");
    fprintf(out, "\"particles\": [\n");
    for (int i = 0; i < N; ++i) dumpParticle(conf.pvec[i], i + 1 < N);
    fprintf(out, "],\n");

    // Ordered pairs passing the prefilter: [i, j, energy, bits, distSq]; the rest are exactly 0.
    long nSkipped = 0;
    fprintf(out, "\"pairs\": [\n");
    bool firstRow = true;
    for (int i = 0; i < N && i < maxI; ++i) {
        ConList con = conf.pvec.getConlist(i);
        for (int j = 0; j < N; ++j) {
            if (i == j) continue;
            double dsq;
            unsigned bits = verdict(&conf.pvec[i], &conf.pvec[j], &con, &dsq);
            double e = pairE(&conf.pvec[i], &conf.pvec[j], &con);
            if (!(bits & V_EVAL)) {
                if (e != 0.0) { fprintf(stderr, "prefiltered pair with nonzero energy\n"); return 1; }
                ++nSkipped;
                continue;
            }
            fprintf(out, "%s[%d, %d, %s, %u, %s]", firstRow ? "" : ",\n", i, j, J(e), bits, J(dsq));
            firstRow = false;
        }
    }
    fprintf(out, "\n],\n\"n_prefiltered\": %ld,\n", nSkipped);

    fprintf(out, "\"one_to_all\": [");
    for (int i = 0; i < N; ++i) fprintf(out, "%s%s", J(oneToAllFresh(pairE, i)), i + 1 < N ? ", " : "");
    fprintf(out, "],\n\"all_to_all\": %s,\n", J(allToAllFresh(pairE)));

    // mol2othersTrial (empty conlist) for every chain.
    fprintf(out, "\"mol2others\": [");
    for (int c = 0; c < conf.pvec.getChainCount(); ++c) {
        Molecule mol = conf.pvec.getChain(c);
        ConList empty;
        double e = 0.0;
        for (unsigned j = 0; j < mol.size(); ++j) {
            for (int i = 0; i < mol[0]; ++i) e += pairE(&conf.pvec[mol[j]], &conf.pvec[i], &empty);
            for (int i = mol.back() + 1; i < N; ++i) e += pairE(&conf.pvec[mol[j]], &conf.pvec[i], &empty);
        }
        fprintf(out, "%s[%d, %d, %s]", c ? ", " : "", mol[0], (int)mol.size(), J(e));
    }
    fprintf(out, "],\n");

    // Scripted trial moves (not accepted: the configuration stays fixed).
    fprintf(out, "\"trials\": [\n");
    for (int t = 0; t < nTrials; ++t) {
        long target = (long)(ran2() * N);
        Particle orig = conf.pvec[target];
        int g = topo.ia_params[orig.type][orig.type].geotype[0];
        double eOld = oneToAllFresh(pairE, (int)target);
        bool displace = (ran2() < 0.5) || g >= SP;
        Vector dr(0, 0, 0), axis(0, 0, 0);
        double angle = 0.0;
        int cw = 0;
        if (displace) {
            double mx = sim.stat.trans[orig.type].mx;
            if (mx == 0.0) mx = 0.2;
            dr.randomUnitSphere();
            dr.x *= mx / conf.geo.box.x; dr.y *= mx / conf.geo.box.y; dr.z *= mx / conf.geo.box.z;
            conf.pvec[target].pos.x += dr.x; conf.pvec[target].pos.y += dr.y; conf.pvec[target].pos.z += dr.z;
        } else {
            double amax = sim.stat.rot[orig.type].angle;
            if (amax == 0.0) amax = 0.3;
            angle = amax * ran2();
            axis = Vector::getRandomUnitSphere();
            cw = (ran2() < 0.5) ? 1 : 0;
            conf.pvec[target].pscRotate(angle, g, axis, cw);
            conf.pvec[target].patchdir[0].ortogonalise(conf.pvec[target].dir);
        }
        double eNew = oneToAllFresh(pairE, (int)target);
        fprintf(out, "{\"target\": %ld, \"displace\": %d, ", target, (int)displace);
        pv("dr", dr); pv("axis", axis);
        fprintf(out, "\"angle\": %s, \"cw\": %d, \"e_old\": %s, \"e_new\": %s, \"state\": ", J(angle), cw, J(eOld), J(eNew));
        dumpParticle(conf.pvec[target], false);
        fprintf(out, "}%s\n", t + 1 < nTrials ? "," : "");
        conf.pvec[target] = orig;
    }
    fprintf(out, "],\n");

    // Wang-Landau: the reference's own WangLandau::init on this configuration (starting
    // bins, system centre) and WangLandau::write of the weights it read (wanglandau.cpp).
    if (sim.wlm[0] > 0 && access(files.wlinfile, R_OK) == 0) {
        fflush(stdout);
        int keep = dup(1);
        dup2(2, 1);
        WangLandau wl(&conf, &sim);
        wl.init(files.wlinfile);
        wl.write((char*)"wl-ref-written.dat");
        fflush(stdout);
        dup2(keep, 1);
        fprintf(out, "\"wl\": {\"currorder\": [%ld, %ld], \"length\": [%ld, %ld], \"alpha\": %s, ", wl.currorder[0],
                wl.currorder[1], wl.length[0], wl.length[1], J(wl.alpha));
        fprintf(out, "\"minorder\": [%s, %s], \"dorder\": [%s, %s], \"sysvolume\": %s, ", J(wl.minorder[0]),
                J(wl.minorder[1]), J(wl.dorder[0]), J(wl.dorder[1]), J(conf.sysvolume));
        pv("syscm", conf.syscm);
        fprintf(out, "\"written\": \"");
        FILE* wf = fopen("wl-ref-written.dat", "r");
        for (int ch; wf && (ch = fgetc(wf)) != EOF;) {
            if (ch == '\n') fprintf(out, "\\n");
            else fputc(ch, out);
        }
        if (wf) fclose(wf);
        fprintf(out, "\"},\n");
    }

    // Isotropic volume trials: box edges += psch (movecreator.cpp:390-421).
    fprintf(out, "\"volume_trials\": [");
    double psch_list[2] = {-0.02 * conf.geo.box.x, 0.015 * conf.geo.box.x};
    for (int k = 0; k < 2; ++k) {
        Vector box0 = conf.geo.box;
        conf.geo.box.x += psch_list[k]; conf.geo.box.y += psch_list[k]; conf.geo.box.z += psch_list[k];
        double e = allToAllFresh(pairE);
        fprintf(out, "%s{\"psch\": %s, \"e_new\": %s}", k ? ", " : "", J(psch_list[k]), J(e));
        conf.geo.box = box0;
    }
    fprintf(out, "],\n\"n\": %d\n}\n", N);
    return 0;
}
