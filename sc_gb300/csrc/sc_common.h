// sc_common.h -- types shared by the host library and the CUDA kernels.
//
// Geometric type codes and the interaction-functor table follow the reference:
// scOOP/structures/macros.h:70-85 (type codes) and scOOP/mc/paire.cpp:6-80
// (which pair functor handles which pair of geometric types).
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define SC_HD __host__ __device__ __forceinline__
#else
#define SC_HD inline
#endif

namespace scg {

constexpr int MAXT = 40;      // type numbers 0..39 (macros.h:78)
constexpr int MAXMT = 100;    // molecule types (macros.h:79)
constexpr int MAXCHL = 20;    // longest chain (macros.h:62)
constexpr int MAX_DEV_TYPES = 16;   // distinct particle types one system may use on the device

enum Geo : int { SCN = 10, SCA = 11, PSC = 12, CPSC = 13, CHPSC = 14, CHCPSC = 15, TPSC = 16, TCPSC = 17,
                 TCHPSC = 18, TCHCPSC = 19, SP = 30, SPN = 30, SPA = 31 };

// Pair functor selected by PairE::initIntFCE for a (geotype, geotype) pair.
enum Kind : int { K_NONE = 0, K_SC_PSC_CPSC, K_SC_CPSC, K_SC_PSC, K_SC_SCN, K_SC_SCA,
                  K_SP_WCA, K_SP_SPA, K_MIX_SCA_SPA, K_MIX_PSC_SP, K_MIX_CPSC_SP };

// Verdict bits reported per evaluated pair.
enum : unsigned { V_EVAL = 1u << 0, V_WCA = 1u << 1, V_ATR = 1u << 2, V_FAR = 1u << 3 };

SC_HD bool isPscFamily(int g) { return g == PSC || g == CHPSC || g == TPSC || g == TCHPSC; }
SC_HD bool isCpscFamily(int g) { return g == CPSC || g == CHCPSC || g == TCPSC || g == TCHCPSC; }
SC_HD bool isTwoPatch(int g) { return g == TPSC || g == TCPSC || g == TCHPSC || g == TCHCPSC; }
SC_HD bool isChiral(int g) { return g == CHPSC || g == CHCPSC || g == TCHPSC || g == TCHCPSC; }

// The functor table of PairE::initIntFCE; later rules override earlier ones there too.
SC_HD int functorKind(int g, int o) {
    int k = K_NONE;
    if ((isCpscFamily(g) && isPscFamily(o)) || (isPscFamily(g) && isCpscFamily(o))) k = K_SC_PSC_CPSC;
    if (isCpscFamily(g) && isCpscFamily(o)) k = K_SC_CPSC;
    if (isPscFamily(g) && isPscFamily(o)) k = K_SC_PSC;
    if (g == SCN && o == SCN) k = K_SC_SCN;
    if (g == SCA && o == SCA) k = K_SC_SCA;
    if (g == SPN || o == SPN) k = K_SP_WCA;
    if (g == SPA && o == SPA) k = K_SP_SPA;
    if ((g == SCA && o == SPA) || (g == SPA && o == SCA)) k = K_MIX_SCA_SPA;
    if ((isPscFamily(g) && (o == SPA || o == SPN)) || ((g == SPA || g == SPN) && isPscFamily(o))) k = K_MIX_PSC_SP;
    if ((isCpscFamily(g) && (o == SPA || o == SPN)) || ((g == SPA || g == SPN) && isCpscFamily(o))) k = K_MIX_CPSC_SP;
    return k;
}

// One entry of the interaction table as the kernels read it: the subset of the
// reference's Ia_param (scOOP/structures/structures.h:187-254) that the pair
// energy uses, plus the functor kind and the patch-combination flags that
// getGeoTypes would derive at every call (paire.h:486-497, 674-685, 891-906, 981-1005).
struct PairParam {
    int geotype[2];
    int kind;
    int exclude;
    int fCH, sCH, fT, sT;          // SC-SC: chiral / two-patch flags of each side
    int firstPsc, secondPsc;       // SC-SC: which intersection routine each side uses
    int mixChiral, mixSec;         // SC-sphere (entry with the SC first): chiral / second patch
    double sigma, epsilon, A, B, pdis, pswitch, pswitchINV;
    double pcangl[4], pcanglsw[4];
    double rcut, rcutSq, rcutwca, rcutwcaSq;
    double half_len[2];
    double parallel;
    // Exact-zero screen used by the move kernels: the pair energy is exactly 0 when the
    // closest segment (SC-SC) or point-segment (SC-sphere) distance^2 exceeds screenSq
    // and the pair is not bonded (the repulsive and attractive branches are both off).
    int screen;        // 0: none (spheres), 1: segment-segment, 2: point-segment, 3: always zero
    int scFirst;       // SC-sphere: 1 if the first particle is the spherocylinder
    int simple;        // SC-SC pair of patchy types (PSC / CPSC families): evaluated as parallel chains
    int pad2_;
    double screenSq;
    double scHalf;     // SC-sphere: half length of the spherocylinder
};

// Bond / angle constants of a molecule type (scOOP/structures/moleculeparams.h:10-79),
// resolved into the ConList fields of ParticleVector::getConlist (Conf.h:97-146).
struct MolParam {
    int size;
    int bonded;       // first-neighbour bond present (bond1 / bondd / bondh)
    int bonded2;      // second-neighbour bond present (bond2)
    int pad_;
    double eq0, c0, mod0, mod1, sp;   // ConList eq[0], c[0], mod[0], mod[1], sp
    double eq1, c1;                   // ConList eq[1], c[1]
    double angle1c, angle1eq, angle2c, angle2eq;
};

// Orientation vectors of one particle beyond its axis.
struct PatchSet {
    double pd[2][3];   // patchdir[0..1]
    double ps[4][3];   // patchsides[0..3]
    double ch[2][3];   // chdir[0..1]
};

}  // namespace scg
