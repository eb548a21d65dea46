// sc_oracle.cpp -- CPU oracle (TEST INFRASTRUCTURE ONLY; see sc_oracle.h).
//
// A plain restatement of the reference's arithmetic in the reference's own
// operation order, so that verdicts come out bit-identical when compiled
// without FMA contraction (-ffp-contract=off).  Every function names the
// reference code it follows (paths relative to the robertvacha/SC tree).

#include "sc_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

const double kPI = 3.141592653589793238462643383279;   // scOOP/structures/macros.h:63
const double kPIH = 1.57079632679489661923132169163975;
enum { SCN = 10, SCA = 11, PSC = 12, CPSC = 13, CHPSC = 14, CHCPSC = 15, TPSC = 16, TCPSC = 17,
       TCHPSC = 18, TCHCPSC = 19, SP = 30, SPN = 30, SPA = 31 };

inline or_vec V(double x, double y, double z) { or_vec v; v.x = x; v.y = y; v.z = z; return v; }
inline double dot(const or_vec& a, const or_vec& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline or_vec scale(double s, const or_vec& v) { return V(v.x * s, v.y * s, v.z * s); }
inline or_vec neg(const or_vec& v) { return V(-1.0 * v.x, -1.0 * v.y, -1.0 * v.z); }
// Vector::size() (scOOP/structures/Vector.h:49-51); gcc folds pow(x,2) into x*x.
inline double vsize(const or_vec& v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
// vecCrossProduct (scOOP/mc/math_calc.h:40-42)
inline or_vec cross(const or_vec& A, const or_vec& B) {
    return V(A.y * B.z - A.z * B.y, -A.x * B.z + A.z * B.x, A.x * B.y - A.y * B.x);
}
// Vector::perpProject (Vector.h:266-277)
inline or_vec perp(const or_vec& a, const or_vec& B) {
    double dp = dot(a, B);
    return V(a.x - B.x * dp, a.y - B.y * dp, a.z - B.z * dp);
}
// Vector::normalise (Vector.h:57-65)
inline void normalise(or_vec& v) {
    double tot = vsize(v);
    if (tot != 0.0) { tot = 1.0 / tot; v.x *= tot; v.y *= tot; v.z *= tot; }
}
// Vector::ortogonalise (Vector.h:128-130)
inline void ortho(or_vec& a, const or_vec& B) {
    double dp = dot(a, B);
    a.x -= dp * B.x; a.y -= dp * B.y; a.z -= dp * B.z;
}
// Vector::rotate(axis, cos, sin) (Vector.h:133-157)
inline void rotate(or_vec& v, const or_vec& axis, double c, double s) {
    double qw = c, qx = axis.x * s, qy = axis.y * s, qz = axis.z * s;
    double t2 = qw * qx, t3 = qw * qy, t4 = qw * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
           t9 = qy * qz, t10 = -qz * qz;
    double nx = 2.0 * ((t8 + t10) * v.x + (t6 - t4) * v.y + (t3 + t7) * v.z) + v.x;
    double ny = 2.0 * ((t4 + t6) * v.x + (t5 + t10) * v.y + (t9 - t2) * v.z) + v.y;
    double nz = 2.0 * ((t7 - t3) * v.x + (t2 + t9) * v.y + (t5 + t8) * v.z) + v.z;
    v.x = nx; v.y = ny; v.z = nz;
}

// Round-half-even of |d| < 2^31, the value Cuboid::image gets from the low word
// of d + 1.5*2^52 (scOOP/structures/geometry.h:110-128).
inline double anint(double d) {
    const double tt = d + 6755399441055744.0;
    uint64_t bits;
    std::memcpy(&bits, &tt, 8);
    return (double)(int32_t)(uint32_t)(bits & 0xffffffffu);
}
inline or_vec image(const or_vec& r1, const or_vec& r2, const double* box) {
    double dx = r1.x - r2.x, dy = r1.y - r2.y, dz = r1.z - r2.z;
    return V(box[0] * (dx - anint(dx)), box[1] * (dy - anint(dy)), box[2] * (dz - anint(dz)));
}

inline bool isPscF(int g) { return g == PSC || g == CHPSC || g == TPSC || g == TCHPSC; }
inline bool isCpscF(int g) { return g == CPSC || g == CHCPSC || g == TCPSC || g == TCHCPSC; }
inline bool isTF(int g) { return g == TPSC || g == TCPSC || g == TCHPSC || g == TCHCPSC; }
inline bool isCHF(int g) { return g == CHPSC || g == CHCPSC || g == TCHPSC || g == TCHCPSC; }

enum Kind { K_NONE = 0, K_SC_PSC_CPSC, K_SC_CPSC, K_SC_PSC, K_SC_SCN, K_SC_SCA,
            K_SP_WCA, K_SP_SPA, K_MIX_SCA_SPA, K_MIX_PSC_SP, K_MIX_CPSC_SP };

// Functor table of PairE::initIntFCE (scOOP/mc/paire.cpp:6-80); later rules override earlier ones.
int functorKind(int g, int o) {
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

// ConList (scOOP/structures/Conf.h:17-33) by particle index; -1 = none.
struct Con {
    bool isEmpty = true;
    double sp = 0.0, mod[2] = {0.0, 0.0}, c[2] = {0.0, 0.0}, eq[2] = {0.0, 0.0};
    int idx[4] = {-1, -1, -1, -1};
};

// ParticleVector::getConlist (scOOP/structures/Conf.h:90-147).
Con getConlist(const or_system* s, int i) {
    Con con;
    const or_particle& p = s->p[i];
    const or_moltype& m = s->mols[p.molType];
    if (m.size == 1) return con;
    int pos = (i - m.first) % m.size;
    if (m.bond1c >= 0.0 || m.bonddc >= 0.0 || m.bondhc >= 0.0) {
        if (pos > 0) con.idx[0] = i - 1;
        if (pos + 1 < m.size) con.idx[1] = i + 1;
        if (m.bond1c >= 0.0) { con.eq[0] = m.bond1eq; con.c[0] = m.bond1c; con.mod[0] = 0.0; con.mod[1] = 0.0; con.sp = 0.0; }
        if (m.bonddc >= 0.0) { con.eq[0] = 0.0; con.c[0] = m.bonddc; con.mod[0] = m.bonddeq; con.mod[1] = 0.0; con.sp = 0.0; }
        if (m.bondhc >= 0.0) { con.eq[0] = 0.0; con.c[0] = m.bondhc; con.mod[0] = m.bondheq; con.mod[1] = m.bondheq; con.sp = m.bondheq; }
        con.isEmpty = false;
    }
    if (m.bond2c >= 0.0) {
        if (pos > 1) con.idx[2] = i - 2;
        if (pos + 2 < m.size) con.idx[3] = i + 2;
        con.eq[1] = m.bond2eq; con.c[1] = m.bond2c;
        con.isEmpty = false;
    }
    return con;
}

// EBond::harmonicPotential (scOOP/mc/paire.h:202-204)
inline double harmonic(double a, double eq, double k) { return k * (a - eq) * (a - eq) * 0.5; }

// fanglScale (scOOP/mc/paire.h:12-17)
inline double fangl(double a, double pcangl, double pcanglsw) {
    if (a <= pcanglsw) return 0.0;
    return (a >= pcangl) ? 1.0 : (0.5 - ((pcanglsw + pcangl) * 0.5 - a) / (pcangl - pcanglsw));
}

// EPatch::minDistSegments (scOOP/mc/paire.cpp:85-241)
or_vec minDistSegments(const or_vec& segA, const or_vec& segB, double halfl1, double halfl2, const or_vec& r_cm) {
    or_vec u = scale(2.0 * halfl1, segA), v = scale(2.0 * halfl2, segB), w, vec;
    double a, b, c, d, e, D, sc, sN, sD, tc, tN, tD;
    bool par = false;
    w.x = segB.x * halfl2 - segA.x * halfl1 - r_cm.x;
    w.y = segB.y * halfl2 - segA.y * halfl1 - r_cm.y;
    w.z = segB.z * halfl2 - segA.z * halfl1 - r_cm.z;
    a = dot(u, u); b = dot(u, v); c = dot(v, v); d = dot(u, w); e = dot(v, w);
    D = a * c - b * b;
    sc = sN = sD = D; tc = tN = tD = D;
    if (D < 0.00000001) {
        par = true; sN = 0.0; sD = 1.0; tN = e; tD = c;
    } else {
        sN = (b * e - c * d); tN = (a * e - b * d);
        if (sN < 0.0) { sN = 0.0; tN = e; tD = c; }
        else if (sN > sD) { sN = sD; tN = e + b; tD = c; }
    }
    if (tN < 0.0) {
        tN = 0.0;
        if (-d < 0.0) sN = 0.0;
        else if (-d > a) sN = sD;
        else { sN = -d; sD = a; }
    } else if (tN > tD) {
        tN = tD;
        if ((-d + b) < 0.0) sN = 0;
        else if ((-d + b) > a) sN = sD;
        else { sN = (-d + b); sD = a; }
    }
    sc = (fabs(sN) < 0.00000001) ? 0.0 : sN / sD;
    tc = (fabs(tN) < 0.00000001) ? 0.0 : tN / tD;
    vec.x = u.x * sc + w.x - v.x * tc;
    vec.y = u.y * sc + w.y - v.y * tc;
    vec.z = u.z * sc + w.z - v.z * tc;
    if (par) {
        or_vec vec2;
        w.x = segA.x * halfl1 - segB.x * halfl2 + r_cm.x;
        w.y = segA.y * halfl1 - segB.y * halfl2 + r_cm.y;
        w.z = segA.z * halfl1 - segB.z * halfl2 + r_cm.z;
        d = dot(v, w); e = dot(u, w);
        D = a * c - b * b;
        sc = sN = sD = D; tc = tN = tD = D;
        if (D < 0.00000001) { sN = 0.0; sD = 1.0; tN = e; tD = a; }
        if (tN < 0.0) {
            tN = 0.0;
            if (-d < 0.0) sN = 0.0;
            else if (-d > c) sN = sD;
            else { sN = -d; sD = c; }
        } else if (tN > tD) {
            tN = tD;
            if ((-d + b) < 0.0) sN = 0;
            else if ((-d + b) > c) sN = sD;
            else { sN = (-d + b); sD = c; }
        }
        sc = (fabs(sN) < 0.00000001) ? 0.0 : sN / sD;
        tc = (fabs(tN) < 0.00000001) ? 0.0 : tN / tD;
        vec2.x = v.x * sc + w.x - u.x * tc;
        vec2.y = v.y * sc + w.y - u.y * tc;
        vec2.z = v.z * sc + w.z - u.z * tc;
        if (dot(vec2, vec2) < dot(vec, vec)) return vec2;
    }
    return vec;
}

struct PatchV { or_vec dir, s0, s1; };

// EPatch::testIntrPatch (scOOP/mc/paire.h:86-101)
inline void testIntrPatch(const or_vec& dir, const or_vec& patchdir, or_vec vec, double cospatch, double ti, double* in) {
    vec = perp(vec, dir);
    if (dot(patchdir, vec) >= cospatch * vsize(vec)) {
        if (in[0] == 0) { in[0] = ti; return; }
        if (in[1] == 0 && in[0] != ti) { in[1] = ti; return; }
    }
}

// EPatch::scToInfiIntr (paire.h:103-119)
inline void scToInfiIntr(const or_vec& d1, const or_vec& d2, const PatchV& P, const or_vec& r_cm, double pcanglsw,
                         double halfl1, double halfl2, double* in, double x1) {
    if ((x1 >= halfl2) || (x1 <= -halfl2)) return;
    or_vec v1 = V(d2.x * x1 - r_cm.x, d2.y * x1 - r_cm.y, d2.z * x1 - r_cm.z);
    double e = dot(d1, v1);
    if ((e >= halfl1) || (e <= -halfl1)) return;
    testIntrPatch(d1, P.dir, v1, pcanglsw, x1, in);
}

// EPatch::testIntrAtC (paire.h:121-148)
void testIntrAtC(const or_vec& d1, const or_vec& d2, const PatchV& P, const or_vec& r_cm, double pcanglsw, double rcutSq,
                 double halfl1, double halfl2, double* in) {
    or_vec v1 = cross(neg(r_cm), d1), v2 = cross(d2, d1);
    double a = dot(v2, v2), b = 2 * dot(v1, v2), c = -rcutSq + dot(v1, v1), d = b * b - 4 * a * c;
    if (d >= 0) {
        d = sqrt(d);
        a = 0.5 / a;
        double x1 = (-b + d) * a;
        scToInfiIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, x1);
        if (d > 0) {
            x1 = (-b - d) * a;
            scToInfiIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, x1);
        }
    }
}

// EPatch::findIntersectPlaneUni (paire.h:150-181)
bool findIntersectPlaneUni(const or_vec& dirA, const or_vec& dirB, double halfl, const or_vec& r_cm, const or_vec& w_vec,
                           double cospatch, double& ti, double& c, double& d) {
    or_vec nplane = cross(dirA, w_vec);
    double a = dot(nplane, dirB);
    c = 1.0; d = 1.0;
    if (a == 0.0) return false;
    ti = dot(nplane, r_cm) / a;
    if ((ti > halfl) || (ti < -halfl)) return false;
    or_vec dv = V(ti * dirB.x - r_cm.x, ti * dirB.y - r_cm.y, ti * dirB.z - r_cm.z);
    c = dot(dv, w_vec);
    if (c * cospatch < 0) return false;
    d = fabs(dot(dv, dirA)) - halfl;
    return true;
}

// Psc::scToEndSpIntr / calcIntersections / testIntrA (paire.h:588-652)
inline void scToEndSpIntr(const or_vec& d1, const or_vec& d2, const PatchV& P, const or_vec& r_cm, double pcanglsw,
                          double halfl1, double halfl2, double* in, double x1) {
    if ((x1 >= halfl2) || (x1 <= -halfl2)) return;
    or_vec v1 = V(d2.x * x1 - r_cm.x, d2.y * x1 - r_cm.y, d2.z * x1 - r_cm.z);
    double e = dot(d1, v1);
    if ((e >= halfl1) || (e <= -halfl1)) testIntrPatch(d1, P.dir, v1, pcanglsw, x1, in);
}
inline void calcIntersections(const or_vec& d1, const or_vec& d2, const PatchV& P, const or_vec& r_cm, double* in,
                              double pcanglsw, double halfl1, double halfl2, double b, double c) {
    double d = b * b - 4 * c;
    if (d >= 0) {
        d = sqrt(d);
        c = (-b + d) * 0.5;
        scToEndSpIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, c);
        if (d > 0) {
            c = (-b - d) * 0.5;
            scToEndSpIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, c);
        }
    }
}
inline void testIntrA(const or_vec& d1, const or_vec& d2, const PatchV& P, const or_vec& r_cm, double pcanglsw,
                      double rcutSq, double halfl1, double halfl2, double* in) {
    or_vec v1 = V(d2.x * halfl2 - r_cm.x, d2.y * halfl2 - r_cm.y, d2.z * halfl2 - r_cm.z);
    double a = dot(v1, d1);
    or_vec v2 = V(v1.x - d1.x * a, v1.y - d1.y * a, v1.z - d1.z * a);
    double b = dot(v2, v2), d = fabs(a) - halfl1, c;
    if (d <= 0) c = b; else c = d * d + b;
    if (c < rcutSq) testIntrPatch(d1, P.dir, v1, pcanglsw, halfl2, in);
}

// Psc::pscIntersect (paire.h:499-583)
int pscIntersect(const or_vec& d1, const or_vec& d2, const PatchV& P, const or_vec& r_cm, double& in1, double& in2,
                 double pcanglsw, double rcutSq, double halfl1, double halfl2) {
    double c, d, ti, disti;
    double in[2] = {0, 0};
    if (findIntersectPlaneUni(d1, d2, halfl2, r_cm, P.s0, pcanglsw, ti, c, d)) {
        disti = (d <= 0) ? c * c : d * d + c * c;
        if (disti <= rcutSq) in[0] = ti;
    }
    if (findIntersectPlaneUni(d1, d2, halfl2, r_cm, P.s1, pcanglsw, ti, c, d)) {
        disti = (d <= 0) ? c * c : d * d + c * c;
        if (disti <= rcutSq) {
            if (in[0] == 0.0) in[0] = ti;
            else if (ti != in[0]) in[1] = ti;
        }
    }
    if (in[1] != 0.0) { in1 = in[0]; in2 = in[1]; return 2; }
    testIntrAtC(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, halfl2, in);
    if (in[1] == 0.0) {
        or_vec v1 = V(d1.x * halfl1 - r_cm.x, d1.y * halfl1 - r_cm.y, d1.z * halfl1 - r_cm.z);
        or_vec v2 = V(-d1.x * halfl1 - r_cm.x, -d1.y * halfl1 - r_cm.y, -d1.z * halfl1 - r_cm.z);
        calcIntersections(d1, d2, P, r_cm, in, pcanglsw, halfl1, halfl2, 2.0 * dot(v1, d2), dot(v1, v1) - rcutSq);
        calcIntersections(d1, d2, P, r_cm, in, pcanglsw, halfl1, halfl2, 2.0 * dot(v2, d2), dot(v2, v2) - rcutSq);
    } else {
        in1 = in[0]; in2 = in[1]; return 2;
    }
    if (in[1] == 0.0) {
        testIntrA(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, halfl2, in);
        if (in[1] == 0.0) testIntrA(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, -halfl2, in);
    }
    in1 = in[0]; in2 = in[1];
    return (in[1] == 0.0) ? 0 : 2;
}

// CPsc::cpscIntersect (paire.h:687-826)
int cpscIntersect(const or_vec& d1, const or_vec& d2, const PatchV& P, const or_vec& r_cm, double& in1, double& in2,
                  double pcanglsw, double rcutSq, double halfl1, double halfl2) {
    double a, b, c, d, x1, x2, disti, ti;
    double in[2] = {0, 0};
    or_vec v1, v2;
    if (findIntersectPlaneUni(d1, d2, halfl2, r_cm, P.s0, pcanglsw, ti, c, d)) {
        if (d <= 0) { disti = c * c; if (disti <= rcutSq) in[0] = ti; }
    }
    if (findIntersectPlaneUni(d1, d2, halfl2, r_cm, P.s1, pcanglsw, ti, c, d)) {
        if (d <= 0) {
            disti = c * c;
            if (disti <= rcutSq) {
                if (in[0] == 0.0) in[0] = ti;
                else if (ti != in[0]) in[1] = ti;
            }
        }
    }
    if (in[1] != 0.0) { in1 = in[0]; in2 = in[1]; return 2; }
    testIntrAtC(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, halfl2, in);
    if (in[1] == 0.0) {
        a = dot(d1, d2);
        if (a != 0.0) {
            v1 = V(r_cm.x + halfl1 * d1.x, r_cm.y + halfl1 * d1.y, r_cm.z + halfl1 * d1.z);
            x1 = dot(d1, v1) / a;
            if (!((x1 > halfl2) || (x1 < -halfl2))) {
                v2 = V(x1 * d2.x - v1.x, x1 * d2.y - v1.y, x1 * d2.z - v1.z);
                b = dot(v2, v2);
                if (!(b > rcutSq)) testIntrPatch(d1, P.dir, v2, pcanglsw, x1, in);
            }
            v1 = V(r_cm.x - halfl1 * d1.x, r_cm.y - halfl1 * d1.y, r_cm.z - halfl1 * d1.z);
            x2 = dot(d1, v1) / a;
            if (!((x2 > halfl2) || (x2 < -halfl2))) {
                v2 = V(x2 * d2.x - v1.x, x2 * d2.y - v1.y, x2 * d2.z - v1.z);
                b = dot(v2, v2);
                if (!(b > rcutSq)) testIntrPatch(d1, P.dir, v2, pcanglsw, x2, in);
            }
        }
    } else {
        in1 = in[0]; in2 = in[1]; return 2;
    }
    if (in[1] == 0.0) {
        v1 = V(d2.x * halfl2 - r_cm.x, d2.y * halfl2 - r_cm.y, d2.z * halfl2 - r_cm.z);
        a = dot(v1, d1);
        v2 = V(v1.x - d1.x * a, v1.y - d1.y * a, v1.z - d1.z * a);
        b = dot(v2, v2);
        d = fabs(a) - halfl1;
        if (d <= 0) { if (b < rcutSq) testIntrPatch(d1, P.dir, v1, pcanglsw, halfl2, in); }
        if (in[1] == 0.0) {
            v1 = V(-d2.x * halfl2 - r_cm.x, -d2.y * halfl2 - r_cm.y, -d2.z * halfl2 - r_cm.z);
            a = dot(v1, d1);
            v2 = V(v1.x - d1.x * a, v1.y - d1.y * a, v1.z - d1.z * a);
            b = dot(v2, v2);
            d = fabs(a) - halfl1;
            if (d <= 0) { if (b < rcutSq) testIntrPatch(d1, P.dir, v1, pcanglsw, -1.0 * halfl2, in); }
        }
    }
    in1 = in[0]; in2 = in[1];
    return (in[1] == 0.0) ? 0 : 2;
}

// EPatch::atrE (scOOP/mc/paire.cpp:243-301)
double atrE(const or_param& ia, const or_vec& d1, const or_vec& d2, const PatchV& P1, const PatchV& P2, const or_vec& r_cm,
            int pn1, int pn2, double S1, double S2, double T1, double T2) {
    double v1 = fabs(S1 - S2), v2 = fabs(T1 - T2), f0 = 0.5 * (v1 + v2);
    or_vec a1 = scale((S1 + S2) * 0.5, d1), a2 = scale((T1 + T2) * 0.5, d2);
    or_vec vi = V(a2.x - a1.x - r_cm.x, a2.y - a1.y - r_cm.y, a2.z - a1.z - r_cm.z);
    or_vec md = minDistSegments(d1, d2, v1, v2, vi);
    double ndist = sqrt(dot(md, md)), atr;
    if (ndist < ia.pdis) atr = -ia.epsilon;
    else { atr = cos(kPIH * (ndist - ia.pdis) / ia.pswitch); atr *= -atr * ia.epsilon; }
    or_vec w = perp(vi, d1);
    double a = dot(w, P1.dir) / vsize(w);
    double f1 = fangl(a, ia.pcangl[0 + 2 * pn1], ia.pcanglsw[0 + 2 * pn1]);
    w = perp(neg(vi), d2);
    a = dot(w, P2.dir) / vsize(w);
    double f2 = fangl(a, ia.pcangl[1 + 2 * pn2], ia.pcanglsw[1 + 2 * pn2]);
    double paral = 1.0;
    if (ia.parallel != 0.0) {    // EPatch::scparallel (paire.h:77-84)
        double cosa = dot(d1, d2);
        if ((ia.parallel > 0 && cosa > 0) || (ia.parallel < 0 && cosa < 0)) paral = 1.0 + ia.parallel * cosa;
    }
    atr *= f0 * f1 * f2 * paral;
    return atr;
}

inline const or_param& P(const or_system* s, int a, int b) { return s->params[a * OR_MAXT + b]; }

// HarmonicSc (scOOP/mc/paire.h:239-280)
double harmonicSc(const or_system* s, double dist, int i1, int i2, const Con& con) {
    const or_particle& p1 = s->p[i1];
    const or_particle& p2 = s->p[i2];
    const or_param& ia = P(s, p1.type, p2.type);
    if (i2 == con.idx[1] || i2 == con.idx[0]) {
        bool tail = (i2 == con.idx[0]);
        double h1 = (ia.geotype[0] < SP) ? (ia.half_len[0] + con.mod[tail ? 0 : 1]) * (tail ? 1.0 : -1.0) : con.sp;
        double h2 = (ia.geotype[1] < SP) ? (ia.half_len[1] + con.mod[tail ? 1 : 0]) * (tail ? -1.0 : 1.0) : con.sp;
        or_vec v1 = V(p1.pos.x + (p1.dir.x * h1 / s->box[0]), p1.pos.y + (p1.dir.y * h1 / s->box[1]), p1.pos.z + (p1.dir.z * h1 / s->box[2]));
        or_vec v2 = V(p2.pos.x + (p2.dir.x * h2 / s->box[0]), p2.pos.y + (p2.dir.y * h2 / s->box[1]), p2.pos.z + (p2.dir.z * h2 / s->box[2]));
        v1 = image(v1, v2, s->box);
        return harmonic(sqrt(dot(v1, v1)), con.eq[0], con.c[0]);
    }
    if (i2 == con.idx[2] || i2 == con.idx[3]) return harmonic(dist, con.eq[1], con.c[1]);
    return 0.0;
}

// HarmonicSp (paire.h:221-236)
double harmonicSp(double dist, int i2, const Con& con) {
    if (i2 == con.idx[1] || i2 == con.idx[0]) return harmonic(dist, con.eq[0], con.c[0]);
    if (i2 == con.idx[2] || i2 == con.idx[3]) return harmonic(dist, con.eq[1], con.c[1]);
    return 0.0;
}

// AngleSc::angleEnergyAngle2 (paire.h:340-352)
double angle2of(const or_particle& a, const or_particle& b) {
    or_vec ax = cross(a.dir, b.dir);
    or_vec x1 = cross(a.dir, ax), x2 = cross(b.dir, ax);
    double v1x = dot(x1, a.pd[0]), v1y = dot(ax, a.pd[0]), v2x = dot(x2, b.pd[0]), v2y = dot(ax, b.pd[0]);
    return acos((v1x * v2x + v1y * v2y) / (sqrt((v1x * v1x + v1y * v1y) * (v2x * v2x + v2y * v2y))));
}

// AngleSc (paire.h:283-337)
double angleSc(const or_system* s, int i1, int i2, const Con& con) {
    const or_particle& p1 = s->p[i1];
    const or_particle& p2 = s->p[i2];
    const or_param& ia = P(s, p1.type, p2.type);
    const or_moltype& m = s->mols[p1.molType];
    double e = 0.0;
    bool partner = (i2 == con.idx[0] || i2 == con.idx[1]);
    bool tail = (i2 == con.idx[0]);
    if (m.angle1c >= 0 && partner) {
        or_vec v1, v2;
        if (ia.geotype[0] < SP) v1 = p1.dir;
        else {
            double h = ia.half_len[1] * (tail ? -1.0 : 1.0);
            v1 = V(p2.pos.x + p2.dir.x * h / s->box[0], p2.pos.y + p2.dir.y * h / s->box[1], p2.pos.z + p2.dir.z * h / s->box[2]);
            v1 = image(v1, p1.pos, s->box);
            normalise(v1);
        }
        if (ia.geotype[1] < SP) v2 = p2.dir;
        else {
            double h = ia.half_len[0] * (tail ? 1.0 : -1.0);
            v2 = V(p1.pos.x + p1.dir.x * h / s->box[0], p1.pos.y + p1.dir.y * h / s->box[1], p1.pos.z + p1.dir.z * h / s->box[2]);
            v2 = image(v2, p2.pos, s->box);
            normalise(v2);
        }
        e += harmonic(acos(dot(v1, v2)), m.angle1eq, m.angle1c);
    }
    if (m.angle2c >= 0 && partner) {
        if ((ia.geotype[0] < SP) && (ia.geotype[1] < SP)) {
            double ang = tail ? angle2of(p2, p1) : angle2of(p1, p2);
            e += harmonic(ang, m.angle2eq, m.angle2c);
        }
    }
    return e;
}

// WcaTruncSq (paire.h:385-393)
inline double wcaTruncSq(double distSq, const or_param& ia) {
    if (distSq > ia.rcutwcaSq) return 0.0;
    return ia.epsilon + ia.A * pow(distSq, -6) - ia.B * pow(distSq, -3);
}

// PscSpa / CPscSpa / ScaSpa (paire.h:911-1010): attraction of one patch to a sphere.
double patchToSphere(int kind, double dist, double contt, const or_vec& distvec, const or_param& ia, const or_vec& d1,
                     const PatchV& P1) {
    double atr;
    if (dist < ia.pdis) atr = -ia.epsilon;
    else { atr = cos(kPIH * (dist - ia.pdis) / ia.pswitch); atr *= -atr * ia.epsilon; }
    double a = 0.0;
    if (kind != K_MIX_SCA_SPA) {
        or_vec w = perp(distvec, d1);
        a = dot(w, P1.dir) / vsize(w);
    }
    double halfl = ia.half_len[0];
    double b = sqrt(ia.rcutSq - dist * dist), f0;
    if (contt + b > halfl) f0 = halfl; else f0 = contt + b;
    if (contt - b < -halfl) f0 -= -halfl; else f0 -= contt - b;
    if (kind == K_MIX_SCA_SPA) atr *= f0;
    else atr *= fangl(a, ia.pcangl[0], ia.pcanglsw[0]) * (f0);
    return atr;
}

// MixSpSc::closestDist (paire.h:1077-1093)
inline double mixClosest(const or_vec& rc, const or_vec& d1, double halfl, double& contt, or_vec& dv) {
    contt = dot(d1, rc);
    double d = -halfl;
    if (contt >= halfl) d = halfl;
    else if (contt > -halfl) d = contt;
    dv = V(-rc.x + d1.x * d, -rc.y + d1.y * d, -rc.z + d1.z * d);
    return dot(dv, dv);
}

}  // namespace

double pairEnergyCon(const or_system* s, int i, int j, const Con& con, unsigned* bitsOut, double* distSqOut);

extern "C" {

// PairE::operator() (scOOP/mc/paire.h:1209-1220) with the functor bodies of
// SpheroCylinder (1114-1197), MixSpSc (1014-1094) and Sphere (1099-1109).
double or_pair_energy(const or_system* s, int i, int j, unsigned* bitsOut, double* distSqOut) {
    return pairEnergyCon(s, i, j, getConlist(s, i), bitsOut, distSqOut);
}

}  // extern "C"

// PairE::operator() with the conlist of particle i given (the reference builds it once per
// oneToAllTrial / allToAll row, totalenergycalculator.h:389, 511).
double pairEnergyCon(const or_system* s, int i, int j, const Con& con, unsigned* bitsOut, double* distSqOut) {
    unsigned bits = 0;
    double dsqOut = -1.0;
    const or_particle& p1 = s->p[i];
    const or_particle& p2 = s->p[j];
    or_vec r_cm = image(p1.pos, p2.pos, s->box);
    double dotrcm = dot(r_cm, r_cm);
    double energy = 0.0;
    if (dotrcm > s->sqmaxcut && con.isEmpty) goto done;
    {
        bits |= OR_V_EVAL;
        double dist = sqrt(dotrcm);
        const or_param& ia = P(s, p1.type, p2.type);
        int kind = functorKind(ia.geotype[0], ia.geotype[1]);
        if (kind == K_SC_PSC || kind == K_SC_CPSC || kind == K_SC_PSC_CPSC || kind == K_SC_SCN || kind == K_SC_SCA) {
            double abE = 0.0;
            abE = harmonicSc(s, dist, i, j, con);
            abE += angleSc(s, i, j, con);
            or_vec md = minDistSegments(p1.dir, p2.dir, ia.half_len[0], ia.half_len[1], r_cm);
            double distSq = dot(md, md);
            dsqOut = distSq;
            double rep = wcaTruncSq(distSq, ia);
            if (!(distSq > ia.rcutwcaSq)) bits |= OR_V_WCA;
            double atr = 0.0;
            if (!((distSq > ia.rcutSq) || (ia.epsilon == 0.0) || ia.exclude)) {
                bits |= OR_V_ATR;
                int g0 = ia.geotype[0], g1 = ia.geotype[1];
                bool fCH = false, sCH = false, fT = false, sT = false;
                if (kind == K_SC_PSC) {
                    fCH = (g0 == CHPSC || g0 == TCHPSC); sCH = (g1 == CHPSC || g1 == TCHPSC);
                    fT = (g0 == TPSC || g0 == TCHPSC); sT = (g1 == TPSC || g1 == TCHPSC);
                } else if (kind == K_SC_CPSC) {
                    fCH = (g0 == CHCPSC || g0 == TCHCPSC); sCH = (g1 == CHCPSC || g1 == TCHCPSC);
                    fT = (g0 == TCPSC || g0 == TCHCPSC); sT = (g1 == TCPSC || g1 == TCHCPSC);
                } else if (kind == K_SC_PSC_CPSC) {
                    fCH = isCHF(g0); sCH = isCHF(g1); fT = isTF(g0); sT = isTF(g1);
                }
                for (int c = 0; c < 4; ++c) {
                    int pn1 = c & 1, pn2 = c >> 1;
                    if ((pn1 && !fT) || (pn2 && !sT)) continue;
                    if (kind == K_SC_SCN) continue;  // EPatch::operator() returns 0 (paire.h:58-61)
                    const or_vec& d1 = fCH ? p1.ch[pn1] : p1.dir;
                    const or_vec& d2 = sCH ? p2.ch[pn2] : p2.dir;
                    if (kind == K_SC_SCA) {      // Sca::operator() (paire.h:845-852)
                        or_vec m2 = minDistSegments(d1, d2, ia.half_len[0], ia.half_len[1], r_cm);
                        double dd = sqrt(dot(m2, m2));
                        if (!(dd > ia.rcutwca)) atr += ia.A * pow(dd, -12) - ia.B * pow(dd, -6) + ia.epsilon;
                        continue;
                    }
                    PatchV P1{p1.pd[pn1], p1.ps[2 * pn1], p1.ps[2 * pn1 + 1]};
                    PatchV P2{p2.pd[pn2], p2.ps[2 * pn2], p2.ps[2 * pn2 + 1]};
                    bool firstPsc = (kind == K_SC_PSC) || (kind == K_SC_PSC_CPSC && isPscF(g0));
                    bool secondPsc = (kind == K_SC_PSC) || (kind == K_SC_PSC_CPSC && !isPscF(g0));
                    double T1 = 0, T2 = 0, S1 = 0, S2 = 0;
                    int na = firstPsc ? pscIntersect(d1, d2, P1, r_cm, T1, T2, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1])
                                      : cpscIntersect(d1, d2, P1, r_cm, T1, T2, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1]);
                    if (na < 2) continue;
                    bits |= 1u << (8 + 2 * c);
                    or_vec mr = neg(r_cm);
                    int nb = secondPsc ? pscIntersect(d2, d1, P2, mr, S1, S2, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0])
                                       : cpscIntersect(d2, d1, P2, mr, S1, S2, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0]);
                    if (nb < 2) continue;
                    bits |= 1u << (9 + 2 * c);
                    atr += atrE(ia, d1, d2, P1, P2, r_cm, pn1, pn2, S1, S2, T1, T2);
                }
            }
            energy = abE + rep + atr;
        } else if (kind == K_MIX_SCA_SPA || kind == K_MIX_PSC_SP || kind == K_MIX_CPSC_SP) {
            bool isp1Spc = (ia.geotype[0] < SP);
            const or_particle& spc = isp1Spc ? p1 : p2;
            const or_param& iap = isp1Spc ? P(s, p1.type, p2.type) : P(s, p2.type, p1.type);
            or_vec rc = isp1Spc ? r_cm : neg(r_cm);
            double contt = 0.0, abE = 0.0, rep = 0.0, atr = 0.0;
            or_vec dv;
            double distSq = mixClosest(rc, spc.dir, iap.half_len[0], contt, dv);
            dsqOut = distSq;
            abE = harmonicSc(s, dist, i, j, con);
            abE += angleSc(s, i, j, con);
            if (distSq < iap.rcutwcaSq) { rep = wcaTruncSq(distSq, ia); bits |= OR_V_WCA; }
            bool isFar = (kind == K_MIX_CPSC_SP) && ((contt > iap.half_len[0]) || (contt < -iap.half_len[0]));
            if (isFar) bits |= OR_V_FAR;
            if (!((distSq > iap.rcutSq) || (iap.epsilon == 0.0) || iap.exclude || isFar)) {
                bits |= OR_V_ATR;
                int g0 = iap.geotype[0];
                bool chiral = false, sec = false;
                if (kind == K_MIX_PSC_SP) { chiral = (g0 == CHPSC || g0 == TCHPSC); sec = (g0 == TPSC || g0 == TCHPSC); }
                if (kind == K_MIX_CPSC_SP) { chiral = (g0 == CHCPSC || g0 == TCHCPSC); sec = (g0 == TCPSC || g0 == TCHCPSC); }
                if (chiral) distSq = mixClosest(rc, spc.ch[0], iap.half_len[0], contt, dv);
                double dd = sqrt(distSq);
                if (dd < iap.rcut) {
                    bits |= 1u << 8;
                    PatchV P1{spc.pd[0], spc.ps[0], spc.ps[1]};
                    atr = patchToSphere(kind, dd, contt, dv, iap, chiral ? spc.ch[0] : spc.dir, P1);
                }
                if (sec) {
                    distSq = mixClosest(rc, chiral ? spc.ch[1] : spc.dir, iap.half_len[0], contt, dv);
                    dd = sqrt(distSq);
                    if (dd < iap.rcut) {
                        bits |= 1u << 9;
                        PatchV P2{spc.pd[1], spc.ps[2], spc.ps[3]};
                        atr += patchToSphere(kind, dd, contt, dv, iap, chiral ? spc.ch[1] : spc.dir, P2);
                    }
                }
            }
            energy = abE + rep + atr;
        } else if (kind == K_SP_WCA || kind == K_SP_SPA) {
            dsqOut = dotrcm;
            double bond = harmonicSp(dist, j, con);
            double pot = 0.0;
            if (kind == K_SP_WCA) {      // WcaTrunc (paire.h:376-383)
                if (!(dist > ia.rcutwca)) { pot = ia.A * pow(dist, -12) - ia.B * pow(dist, -6) + ia.epsilon; bits |= OR_V_WCA; }
            } else {                      // WcaCos2Taylor (paire.h:416-439)
                if (!(dist > ia.rcut || ia.epsilon == 0.0 || ia.exclude)) {
                    bits |= OR_V_ATR;
                    double e;
                    if (dist > ia.pdis) {
                        e = kPIH * (dist - ia.pdis) * ia.pswitchINV;
                        e *= e;
                        e = (1 - e + e * e * (1.0 / 3.0) - e * e * e * (2.0 / 45.0) + e * e * e * e * (1.0 / 315.0) -
                             e * e * e * e * e * (2.0 / 14175.0) + e * e * e * e * e * e * (2.0 / 467775.0) -
                             e * e * e * e * e * e * e * (4.0 / 42567525) + e * e * e * e * e * e * e * e * (1.0 / 638512875)) *
                            -ia.epsilon;
                    } else {
                        e = -ia.epsilon;
                    }
                    if (dist > ia.rcutwca) pot = e;
                    else { pot = ia.A * pow(dist, -12) - ia.B * pow(dist, -6); bits |= OR_V_WCA; }
                }
            }
            energy = bond + pot;
        }
        // K_NONE: EBasic returns 0 (paire.h:207-213)
    }
done:
    if (bitsOut) *bitsOut = bits;
    if (distSqOut) *distSqOut = dsqOut;
    return energy;
}

extern "C" {

// TotalEMatrix::oneToAllTrial without pair list (totalenergycalculator.h:383-415): index order.
double or_one_to_all(const or_system* s, int target) {
    double e = 0.0;
    for (int i = 0; i < target; ++i) e += or_pair_energy(s, target, i, nullptr, nullptr);
    for (int i = target + 1; i < s->n; ++i) e += or_pair_energy(s, target, i, nullptr, nullptr);
    return e;
}

// TotalEMatrix::allToAll(EnergyMatrix*) (totalenergycalculator.h:502-521): part1 = i > j.
double or_all_to_all(const or_system* s) {
    double e = 0.0;
    for (int i = 1; i < s->n; ++i) {
        const Con con = getConlist(s, i);
        for (int j = 0; j < i; ++j) e += pairEnergyCon(s, i, j, con, nullptr, nullptr);
    }
    return e;
}

// PairE over a batch of ordered pairs (i[k] with the conlist of i[k]).
void or_pair_energies(const or_system* s, long n, const int* I, const int* J, double* E, unsigned* bits,
                      double* dsq) {
    for (long k = 0; k < n; ++k)
        E[k] = pairEnergyCon(s, I[k], J[k], getConlist(s, I[k]), bits ? &bits[k] : nullptr, dsq ? &dsq[k] : nullptr);
}

// The pairs PairE's prefilter admits (paire.h:1209-1215): ordered (i, j), i a target
// (targets[0..nt), or every particle when targets is NULL), j != i, with the image
// distance^2 <= sqmaxcut or j bonded to i (conlist); at most cap written, *count all.
void or_prefilter_pairs(const or_system* s, int nt, const int* targets, long cap, int* I, int* J, long* count) {
    long c = 0;
    const int ntt = targets ? nt : s->n;
    for (int a = 0; a < ntt; ++a) {
        const int i = targets ? targets[a] : a;
        const Con con = getConlist(s, i);
        for (int j = 0; j < s->n; ++j) {
            if (j == i) continue;
            or_vec r = image(s->p[i].pos, s->p[j].pos, s->box);
            const bool bonded = j == con.idx[0] || j == con.idx[1] || j == con.idx[2] || j == con.idx[3];
            if (dot(r, r) > s->sqmaxcut && !bonded) continue;
            if (c < cap) { I[c] = i; J[c] = j; }
            ++c;
        }
    }
    *count = c;
}

// Nematic order parameter (no counterpart in the reference): S2, the largest eigenvalue of
// Q = <3/2 u u^T - 1/2 I> over the axes of the spherocylinders (geotype < SP), and the
// director, by cyclic Jacobi rotations.
int or_nematic(const or_system* s, double* s2, double dir[3]) {
    double m[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < s->n; ++i) {
        const or_particle& p = s->p[i];
        if (P(s, p.type, p.type).geotype[0] >= SP) continue;
        const or_vec& d = p.dir;
        m[0] += 1.0;
        m[1] += d.x * d.x; m[2] += d.y * d.y; m[3] += d.z * d.z;
        m[4] += d.x * d.y; m[5] += d.x * d.z; m[6] += d.y * d.z;
    }
    if (m[0] < 1.0) { *s2 = 0.0; if (dir) dir[0] = dir[1] = dir[2] = 0.0; return 0; }
    const double n = m[0];
    double a[3][3] = {{1.5 * m[1] / n - 0.5, 1.5 * m[4] / n, 1.5 * m[5] / n},
                      {1.5 * m[4] / n, 1.5 * m[2] / n - 0.5, 1.5 * m[6] / n},
                      {1.5 * m[5] / n, 1.5 * m[6] / n, 1.5 * m[3] / n - 0.5}};
    double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 60; ++sweep) {
        if (a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2] < 1e-30) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (a[p][q] == 0.0) continue;
                const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; ++k) { double x = a[k][p], y = a[k][q]; a[k][p] = c * x - sn * y; a[k][q] = sn * x + c * y; }
                for (int k = 0; k < 3; ++k) { double x = a[p][k], y = a[q][k]; a[p][k] = c * x - sn * y; a[q][k] = sn * x + c * y; }
                for (int k = 0; k < 3; ++k) { double x = v[k][p], y = v[k][q]; v[k][p] = c * x - sn * y; v[k][q] = sn * x + c * y; }
            }
    }
    int b = 0;
    for (int k = 1; k < 3; ++k) if (a[k][k] > a[b][b]) b = k;
    *s2 = a[b][b];
    if (dir) for (int k = 0; k < 3; ++k) dir[k] = v[k][b];
    return 0;
}

// TotalEMatrix::mol2othersTrial (totalenergycalculator.h:453-499): empty conlist.
double or_mol2others(const or_system* s, int first, int size) {
    // An empty conlist is what a moleculeless system would give: evaluate with a
    // copy whose molecule table says "single particles".
    double e = 0.0;
    or_moltype single{};
    single.size = 1;
    std::vector<or_moltype> mols(s->nmol > 0 ? s->nmol : 1, single);
    or_system t = *s;
    t.mols = mols.data();
    for (int j = first; j < first + size; ++j) {
        for (int i = 0; i < first; ++i) e += or_pair_energy(&t, j, i, nullptr, nullptr);
        for (int i = first + size; i < s->n; ++i) e += or_pair_energy(&t, j, i, nullptr, nullptr);
    }
    return e;
}

// Inicializer::fillTypes (scOOP/mc/inicializer.cpp:660-852), Topo::genParamPairs and
// Topo::genTopoParams (scOOP/structures/topo.cpp:5-153).
int or_derive_params(const or_type_in* types, int ntypes, const unsigned char* excl, or_param* ia, double* sqmaxcutOut,
                     double* maxcutOut) {
    std::memset(ia, 0, sizeof(or_param) * OR_MAXT * OR_MAXT);
    double sqmaxcut = 0.0;
    for (int k = 0; k < ntypes; ++k) {
        const or_type_in& t = types[k];
        if (t.type < 0 || t.type >= OR_MAXT) return -1;
        or_param& p = ia[t.type * OR_MAXT + t.type];
        const double* q = t.param;
        int f = t.nfields, g = t.geotype;
        p.geotype[0] = p.geotype[1] = g;
        p.epsilon = q[0];
        p.sigma = q[1];
        p.A = 4 * p.epsilon * pow(p.sigma, 12);
        p.B = 4 * p.epsilon * pow(p.sigma, 6);
        p.rcutwca = (p.sigma) * pow(2.0, 1.0 / 6.0);
        p.rcutwcaSq = p.rcutwca * p.rcutwca;
        if (f > 0 && f != 1 && f != 3) {
            p.pdis = q[2];
            p.pswitch = q[3];
            p.pswitchINV = 1.0 / q[3];
            p.rcut = (g != SPN) ? p.pswitch + p.pdis : 0.0;
            p.rcutSq = p.rcut * p.rcut;
        }
        if (f == 1) for (int i = 0; i < 2; ++i) { p.len[i] = q[2]; p.half_len[i] = q[2] / 2; }
        if (f == 3) for (int i = 0; i < 2; ++i) { p.len[i] = q[4]; p.half_len[i] = q[4] / 2; }
        if (f > 2 && f != 3) {
            for (int i = 0; i < 2; ++i) {
                p.len[i] = q[6]; p.half_len[i] = q[6] / 2;
                p.pcangl[i] = cos(q[4] / 2.0 / 180 * kPI);
                p.pcanglsw[i] = cos((q[4] / 2.0 + q[5]) / 180 * kPI);
                p.pcoshalfi[i] = cos((q[4] / 2.0 + q[5]) / 2.0 / 180 * kPI);
                p.psinhalfi[i] = sqrt(1.0 - p.pcoshalfi[i] * p.pcoshalfi[i]);
                p.parallel = q[7];
            }
        }
        if (f == 7) for (int i = 0; i < 2; ++i) {
            p.chiral_cos[i] = cos(q[8] / 360 * kPI);
            p.chiral_sin[i] = sqrt(1 - p.chiral_cos[i] * p.chiral_cos[i]);
        }
        if (f == 9 || f == 10) for (int i = 0; i < 2; ++i) {
            p.csecpatchrot[i] = cos(q[8] / 360 * kPI);
            p.ssecpatchrot[i] = sqrt(1 - p.csecpatchrot[i] * p.csecpatchrot[i]);
            p.pcangl[i + 2] = cos(q[9] / 2.0 / 180 * kPI);
            p.pcanglsw[i + 2] = cos((q[9] / 2.0 + q[10]) / 180 * kPI);
            p.pcoshalfi[i + 2] = cos((q[9] / 2.0 + q[10]) / 2.0 / 180 * kPI);
            p.psinhalfi[i + 2] = sqrt(1.0 - p.pcoshalfi[i + 2] * p.pcoshalfi[i + 2]);
        }
        if (f == 10) for (int i = 0; i < 2; ++i) {
            p.chiral_cos[i] = cos(q[11] / 360 * kPI);
            p.chiral_sin[i] = sqrt(1 - p.chiral_cos[i] * p.chiral_cos[i]);
        }
        if (g < SP)
            p.volume = 4.0 / 3.0 * kPI * pow((p.sigma) / 2.0, 3.0) + kPI / 2.0 * p.len[0] * pow((p.sigma) / 2.0, 2.0);
        else
            p.volume = 4.0 / 3.0 * kPI * pow((p.sigma) / 2.0, 3.0);
        if (p.rcutwca > sqmaxcut) sqmaxcut = p.rcutwca;
        if (p.rcut > sqmaxcut) sqmaxcut = p.rcut;
    }
    // raw patch angles, needed by the mixed pairs below
    double pangl[OR_MAXT][4] = {}, panglsw[OR_MAXT][4] = {};
    for (int k = 0; k < ntypes; ++k) {
        const or_type_in& t = types[k];
        if (t.nfields > 2 && t.nfields != 3) { pangl[t.type][0] = t.param[4]; panglsw[t.type][0] = t.param[5]; }
        if (t.nfields == 9 || t.nfields == 10) { pangl[t.type][2] = t.param[9]; panglsw[t.type][2] = t.param[10]; }
    }
    double length = 0;
    for (int i = 0; i < OR_MAXT; ++i) {
        for (int j = 0; j < OR_MAXT; ++j) {
            if (i == j) continue;
            const or_param& di = ia[i * OR_MAXT + i];
            const or_param& dj = ia[j * OR_MAXT + j];
            if (dj.geotype[0] == 0 || di.geotype[0] == 0) continue;
            or_param& p = ia[i * OR_MAXT + j];
            int a[2] = {i, j};
            for (int k = 0; k < 2; ++k) {
                const or_param& dk = ia[a[k] * OR_MAXT + a[k]];
                p.geotype[k] = dk.geotype[0];
                p.len[k] = dk.len[0];
                if (dk.len[0] > 0) {
                    if (length == 0) length = dk.len[0];
                    else if (length > 0 && length != dk.len[0]) return -2;   // topo.cpp:25-32
                }
                p.half_len[k] = dk.half_len[0];
                if (p.geotype[k] >= PSC && p.geotype[k] < SP) {
                    double pa = pangl[a[k]][0], ps = panglsw[a[k]][0];
                    p.pcangl[k] = cos(pa / 2.0 / 180 * kPI);
                    p.pcanglsw[k] = cos((pa / 2.0 + ps) / 180 * kPI);
                    p.pcoshalfi[k] = cos((pa / 2.0 + ps) / 2.0 / 180 * kPI);
                    p.psinhalfi[k] = sqrt(1.0 - p.pcoshalfi[k] * p.pcoshalfi[k]);
                }
                if (isCHF(p.geotype[k])) { p.chiral_cos[k] = dk.chiral_cos[0]; p.chiral_sin[k] = dk.chiral_sin[0]; }
                if (isTF(p.geotype[k])) {
                    p.csecpatchrot[k] = dk.csecpatchrot[0];
                    p.ssecpatchrot[k] = dk.ssecpatchrot[0];
                    double pa = pangl[a[k]][2], ps = panglsw[a[k]][2];
                    p.pcangl[k + 2] = cos(pa / 2.0 / 180 * kPI);
                    p.pcanglsw[k + 2] = cos((pa / 2.0 + ps) / 180 * kPI);
                    p.pcoshalfi[k + 2] = cos((pa / 2.0 + ps) / 2.0 / 180 * kPI);
                    p.psinhalfi[k + 2] = sqrt(1.0 - p.pcoshalfi[k + 2] * p.pcoshalfi[k + 2]);
                }
            }
            p.sigma = ((di.sigma + dj.sigma) * 0.5);
            p.epsilon = sqrt(di.epsilon * dj.epsilon);
            p.A = 4 * p.epsilon * pow(p.sigma, 12);
            p.B = 4 * p.epsilon * pow(p.sigma, 6);
            p.pswitch = ((di.pswitch + dj.pswitch) * 0.5);
            p.pswitchINV = 1.0 / p.pswitch;
            p.rcutwca = (p.sigma) * pow(2.0, 1.0 / 6.0);
            p.rcutwcaSq = p.rcutwca * p.rcutwca;
            if ((di.parallel > 0) && (dj.parallel > 0)) p.parallel = sqrt(di.parallel * dj.parallel);
            if ((di.parallel < 0) && (dj.parallel < 0)) p.parallel = -sqrt(di.parallel * dj.parallel);
            p.pdis = (((di.pdis - di.rcutwca) + (dj.pdis - dj.rcutwca)) * 0.5) + p.rcutwca;
            p.rcut = (p.geotype[0] == SPN || p.geotype[1] == SPN) ? 0.0 : p.pswitch + p.pdis;
            p.rcutSq = p.rcut * p.rcut;
            if (p.rcutwca > sqmaxcut) sqmaxcut = p.rcutwca;
            if (p.rcut > sqmaxcut) sqmaxcut = p.rcut;
        }
    }
    for (int i = 0; i < OR_MAXT; ++i)
        for (int j = 0; j < OR_MAXT; ++j) ia[i * OR_MAXT + j].exclude = excl ? excl[i * OR_MAXT + j] : 0;
    double maxlength = 0;
    for (int i = 0; i < OR_MAXT; ++i) if (maxlength < ia[i * OR_MAXT + i].len[0]) maxlength = ia[i * OR_MAXT + i].len[0];
    sqmaxcut += maxlength;
    sqmaxcut *= 1.1;
    *maxcutOut = sqmaxcut;
    *sqmaxcutOut = sqmaxcut * sqmaxcut;
    return 0;
}

// Particle::init (scOOP/structures/particle.cpp:3-79)
void or_particle_init(or_particle* p, const or_param* d) {
    int g = d->geotype[0];
    if (g == SCA || g == SCN) return;
    normalise(p->dir);
    ortho(p->pd[0], p->dir);
    normalise(p->pd[0]);
    if (g == PSC || g == CPSC || g == TPSC || g == TCPSC) {
        p->ps[0] = p->pd[0]; rotate(p->ps[0], p->dir, d->pcoshalfi[0], d->psinhalfi[0]);
        p->ps[1] = p->pd[0]; rotate(p->ps[1], p->dir, d->pcoshalfi[0], -1.0 * d->psinhalfi[0]);
    }
    if (isTF(g)) {
        p->pd[1] = p->pd[0];
        rotate(p->pd[1], p->dir, d->csecpatchrot[0], d->ssecpatchrot[0]);
        ortho(p->pd[1], p->dir);
        normalise(p->pd[1]);
    }
    if (g == TPSC || g == TCPSC) {
        p->ps[2] = p->pd[1]; rotate(p->ps[2], p->dir, d->pcoshalfi[2], d->psinhalfi[2]);
        p->ps[3] = p->pd[1]; rotate(p->ps[3], p->dir, d->pcoshalfi[2], -1.0 * d->psinhalfi[2]);
    }
    if (isCHF(g)) {
        p->ch[0] = p->dir; rotate(p->ch[0], p->pd[0], d->chiral_cos[0], d->chiral_sin[0]);
        p->ps[0] = p->pd[0]; rotate(p->ps[0], p->ch[0], d->pcoshalfi[0], d->psinhalfi[0]);
        p->ps[1] = p->pd[0]; rotate(p->ps[1], p->ch[0], d->pcoshalfi[0], -1.0 * d->psinhalfi[0]);
    }
    if (g == TCHPSC || g == TCHCPSC) {
        p->ch[1] = p->dir; rotate(p->ch[1], p->pd[1], d->chiral_cos[0], d->chiral_sin[0]);
        p->ps[2] = p->pd[1]; rotate(p->ps[2], p->ch[1], d->pcoshalfi[2], d->psinhalfi[2]);
        p->ps[3] = p->pd[1]; rotate(p->ps[3], p->ch[1], d->pcoshalfi[2], -1.0 * d->psinhalfi[2]);
    }
}

// Particle::pscRotate (scOOP/structures/particle.h:182-272); positive selects +sin.
void or_psc_rotate(or_particle* p, int g, double angle, or_vec ax, int positive) {
    double vc = cos(angle);
    double vs = positive ? sqrt(1.0 - vc * vc) : -sqrt(1.0 - vc * vc);
    double qw = vc, qx = ax.x * vs, qy = ax.y * vs, qz = ax.z * vs;
    double t2 = qw * qx, t3 = qw * qy, t4 = qw * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
           t9 = qy * qz, t10 = -qz * qz;
    double d1 = t8 + t10, d2 = t6 - t4, d3 = t3 + t7, d4 = t4 + t6, d5 = t5 + t10, d6 = t9 - t2, d7 = t7 - t3,
           d8 = t2 + t9, d9 = t5 + t8;
    auto rot = [&](or_vec& v) {
        double nx = 2.0 * (d1 * v.x + d2 * v.y + d3 * v.z) + v.x;
        double ny = 2.0 * (d4 * v.x + d5 * v.y + d6 * v.z) + v.y;
        double nz = 2.0 * (d7 * v.x + d8 * v.y + d9 * v.z) + v.z;
        v.x = nx; v.y = ny; v.z = nz;
    };
    rot(p->dir);
    if (g != SCN && g != SCA) {
        int m = isTF(g) ? 2 : 1;
        for (int k = 0; k < m; ++k) { rot(p->pd[k]); rot(p->ps[2 * k]); rot(p->ps[2 * k + 1]); }
    }
    if (isCHF(g)) {
        int m = (g == TCHPSC || g == TCHCPSC) ? 2 : 1;
        for (int k = 0; k < m; ++k) rot(p->ch[k]);
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Sequential Metropolis loop: the reference's Updater::simulate step loop
// (scOOP/mc/updater.cpp:206-230) with particleMove / partDisplace / partRotate
// (movecreator.cpp:11-33, 947-1028), chainMove (305-328, 1075-1392), the volume move of every
// coupling (330-546) and the
// Verlet pair list of genSimplePairList (updater.cpp:484-552, cutoff main.cpp:117-126).
// Used only as the timed CPU baseline; it draws from a splitmix64 stream
// instead of dSFMT, which changes the trajectory but not the algorithm.
namespace {

struct Rng {
    uint64_t s;
    double operator()() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return (z >> 11) * (1.0 / 9007199254740992.0);
    }
};

// MoveCreator::pressureMove's box change for every coupling (movecreator.cpp:349-546), with
// the reference's arithmetic: propose() changes the box and returns the pressure-volume part
// of enermove, p dV - N T ln(V'/V) for the coupling's dV and V'/V (ptype 3 keeps the volume
// and has none); reject() undoes the change as the reference does, by subtracting it again
// (ptype 0 restores the saved edge, ptype 3 re-derives z from the kept volume).
struct BoxTrial {
    int ptype = 1;
    int side = 0;                       // ptype 0: the edge that changed
    double old = 0.0;                   // ptype 0: its length before
    double d[3] = {0.0, 0.0, 0.0};      // the change of each edge
    double pvol = 0.0;                  // ptype 3: the kept volume
    double propose(double* box, const or_mc_opts* o, int N, Rng& rng) {
        ptype = o->ptype;
        d[0] = d[1] = d[2] = 0.0;
        const double NT = (double)N * o->temper;
        switch (ptype) {
        case 0: {           // one edge chosen at random (movecreator.cpp:349-389)
            const double rs = rng();
            side = rs < 1.0 / 3.0 ? 0 : (rs < 2.0 / 3.0 ? 1 : 2);
            const double area = side == 0 ? box[1] * box[2] : (side == 1 ? box[0] * box[2] : box[0] * box[1]);
            old = box[side];
            box[side] += o->edge_mx * (rng() - 0.5);
            return o->press * area * (box[side] - old) - NT * log(box[side] / old);
        }
        case 2: {           // x and y together, z kept (:422-450)
            const double psch = o->edge_mx * (rng() - 0.5);
            const double pv = box[0] * box[1];
            box[0] += psch; box[1] += psch;
            d[0] = d[1] = psch;
            const double pvoln = box[0] * box[1];
            return o->press * box[2] * (pvoln - pv) - NT * log(pvoln / pv);
        }
        case 3: {           // x and y together, z re-derived to keep the volume (:451-477)
            const double psch = o->edge_mx * (rng() - 0.5);
            pvol = box[0] * box[1] * box[2];
            box[0] += psch; box[1] += psch;
            box[2] = pvol / box[0] / box[1];
            d[0] = d[1] = psch;
            return 0.0;
        }
        case 4: {           // x or y (:478-509); the reference's test `if (ran2() - 0.5)` is true
                            // unless the draw is exactly 0.5, so x changes
            const double pv = box[0] * box[1];
            if (rng() - 0.5 != 0.0) d[0] = o->edge_mx * (rng() - 0.5);
            else d[1] = o->edge_mx * (rng() - 0.5);
            box[0] += d[0]; box[1] += d[1];
            const double pvoln = box[0] * box[1];
            return o->press * box[2] * (pvoln - pv) - NT * log(pvoln / pv);
        }
        case 5: {           // y only (:510-539)
            const double pv = box[1];
            d[1] = o->edge_mx * (rng() - 0.5);
            box[1] += d[1];
            const double pvoln = box[1];
            return o->press * box[2] * box[0] * (pvoln - pv) - NT * log(pvoln / pv);
        }
        default: {          // 1: isotropic (:390-421)
            const double psch = o->edge_mx * (rng() - 0.5);
            const double pv = box[0] * box[1] * box[2];
            box[0] += psch; box[1] += psch; box[2] += psch;
            d[0] = d[1] = d[2] = psch;
            const double pvoln = box[0] * box[1] * box[2];
            return o->press * (pvoln - pv) - NT * log(pvoln / pv);
        }
        }
    }
    void reject(double* box) const {
        if (ptype == 0) {
            box[side] = old;
            return;
        }
        box[0] -= d[0]; box[1] -= d[1];
        if (ptype == 3) box[2] = pvol / box[0] / box[1];
        else box[2] -= d[2];
    }
};

or_vec randomUnitSphere(Rng& r) {     // Vector::randomUnitSphere (Vector.h:190-205)
    double a, xi1, xi2;
    do { xi1 = 1.0 - 2.0 * r(); xi2 = 1.0 - 2.0 * r(); a = xi1 * xi1 + xi2 * xi2; } while (a > 1.0);
    double b = 2.0 * sqrt(1.0 - a);
    return V(xi1 * b, xi2 * b, 1.0 - 2.0 * a);
}

// Verlet list of genSimplePairList (updater.cpp:484-552): every pair (i < j) with
// |r_cm|^2 <= cut2 or bonded to i+1 (bond1/bondd/bondh) or i+2 (bond2), both directions,
// neighbours in ascending index order.  Flat storage (start offsets + ids).
struct PairList {
    std::vector<int> start, count, ids;
    void build(const or_system* s, double cut2) {
        const int n = s->n;
        count.assign(n, 0);
        auto bondedPair = [&](int i, int j) {
            if (j > i + 2) return false;
            const or_moltype& m = s->mols[s->p[i].molType];
            int pos = (i - m.first) % m.size;
            if ((m.bond1c >= 0.0 || m.bonddc >= 0.0 || m.bondhc >= 0.0) && pos + 1 < m.size && i + 1 == j) return true;
            if (m.bond2c >= 0.0 && pos + 2 < m.size && i + 2 == j) return true;
            return false;
        };
        std::vector<std::pair<int, int>> pairs;
        pairs.reserve((size_t)n * 64);
        for (int i = 0; i + 1 < n; ++i)
            for (int j = i + 1; j < n; ++j) {
                or_vec r = image(s->p[i].pos, s->p[j].pos, s->box);
                if (dot(r, r) <= cut2 || bondedPair(i, j)) {
                    pairs.emplace_back(i, j);
                    ++count[i];
                    ++count[j];
                }
            }
        start.assign(n + 1, 0);
        for (int i = 0; i < n; ++i) start[i + 1] = start[i] + count[i];
        ids.resize(start[n]);
        std::vector<int> fill(start.begin(), start.end() - 1);
        // pairs are ordered by i then j: particle t receives its j < t neighbours (as the
        // partner of earlier i) before its j > t ones, each in ascending order
        for (auto& pr : pairs) {
            ids[fill[pr.first]++] = pr.second;
            ids[fill[pr.second]++] = pr.first;
        }
    }
};

// Lower-triangular energy matrix of EnergyMatrixF (totalenergycalculator.h:16-128),
// entry (i, j), i > j, at i (i - 1) / 2 + j.
inline size_t emIdx(int i, int j) { return i > j ? (size_t)i * (i - 1) / 2 + j : (size_t)j * (j - 1) / 2 + i; }

}  // namespace

// The sequential loop as a resumable state: or_mc_open does what precedes the reference's
// timed loop (the initial energy, TotalEMatrix::initEM, and the first pair list), or_mc_advance
// runs the next moves of the sweep loop, so that a caller can time the moves alone.
struct or_mc {
    or_system* s;
    or_mc_opts o;
    Rng rng;
    int N;
    double shprob;
    double cut2 = 0.0;
    bool list = false;
    PairList pl;
    bool matrix = false;             // TotalEMatrix (else TotalEFull)
    std::vector<double> em, emTrial, changes;
    double energy = 0.0;
    long sweep = 1;                  // current sweep (1-based, as updater.cpp)
    long step = 1;                   // next step of the current sweep (1..N)
    double setupSeconds = 0.0;
    double swprob = 0.0;             // switchprob when switchable particles exist, else 0
    std::vector<int> switchable;     // the particles with a switch type, in index order
    bool gc = false;                 // grand-canonical moves after every grand_every-th sweep
    std::vector<std::pair<int, int>> chains;                 // (first particle, size) of every chain
    std::vector<std::pair<size_t, double>> chainChanges;     // a chain trial's matrix slots and energies
};

namespace {

// TotalEMatrix::oneToAll / TotalEFull::oneToAll with the pair list (totalenergycalculator.h:
// 355-381, 561-580): the target's old energy from the matrix, or by pair energies.
double mcOld(or_mc& m, int t) {
    double e = 0.0;
    if (m.list) {
        const int* id = m.pl.ids.data() + m.pl.start[t];
        const int cnt = m.pl.count[t];
        if (m.matrix) {
            for (int k = 0; k < cnt; ++k) e += m.em[emIdx(t, id[k])];
        } else {
            const Con con = getConlist(m.s, t);
            for (int k = 0; k < cnt; ++k) e += pairEnergyCon(m.s, t, id[k], con, nullptr, nullptr);
        }
        return e;
    }
    if (m.matrix) {
        for (int i = 0; i < m.N; ++i) if (i != t) e += m.em[emIdx(t, i)];
        return e;
    }
    return or_one_to_all(m.s, t);
}

// oneToAllTrial (:383-415): pair energies of the moved target, kept in `changes`.
double mcTrial(or_mc& m, int t) {
    double e = 0.0;
    const Con con = getConlist(m.s, t);
    if (m.list) {
        const int* id = m.pl.ids.data() + m.pl.start[t];
        const int cnt = m.pl.count[t];
        if (m.matrix) m.changes.resize(cnt);
        for (int k = 0; k < cnt; ++k) {
            double v = pairEnergyCon(m.s, t, id[k], con, nullptr, nullptr);
            if (m.matrix) m.changes[k] = v;
            e += v;
        }
        return e;
    }
    if (m.matrix) m.changes.assign(m.N, 0.0);
    for (int i = 0; i < m.N; ++i) {
        if (i == t) continue;
        double v = pairEnergyCon(m.s, t, i, con, nullptr, nullptr);
        if (m.matrix) m.changes[i] = v;
        e += v;
    }
    return e;
}

// EnergyMatrixF::fixEMatrixSingle (:61-79)
void mcCommit(or_mc& m, int t) {
    if (!m.matrix) return;
    if (m.list) {
        const int* id = m.pl.ids.data() + m.pl.start[t];
        for (int k = 0; k < m.pl.count[t]; ++k) m.em[emIdx(t, id[k])] = m.changes[k];
    } else {
        for (int i = 0; i < m.N; ++i) if (i != t) m.em[emIdx(t, i)] = m.changes[i];
    }
}

// ParticleVector::getChainCount / getChain: the molecules of more than one particle, in
// particle order, as (first particle, size).
void buildChains(or_mc& m) {
    m.chains.clear();
    for (int t = 0; t < m.s->nmol; ++t) {
        const or_moltype& mt = m.s->mols[t];
        if (mt.size < 2) continue;
        for (int k = 0; k < mt.count; ++k) m.chains.emplace_back(mt.first + k * mt.size, mt.size);
    }
    std::sort(m.chains.begin(), m.chains.end());
}

// TotalEMatrix::mol2others / mol2othersTrial (totalenergycalculator.h:417-499) and
// TotalEFull's (:583-619): the chain's pairs, under an empty conlist, with every particle
// outside it, or with its pair-list neighbours outside it.  The old energy reads the matrix;
// a trial keeps each pair energy with its matrix slot for the commit (fixEMatrixChain,
// :81-114).
double mcChain(or_mc& m, int first, int size, bool trial) {
    const int last = first + size - 1;
    const Con none;
    if (trial) m.chainChanges.clear();
    double e = 0.0;
    auto term = [&](int j, int i) {
        if (!trial && m.matrix) {
            e += m.em[emIdx(j, i)];
            return;
        }
        const double v = pairEnergyCon(m.s, j, i, none, nullptr, nullptr);
        if (trial && m.matrix) m.chainChanges.emplace_back(emIdx(j, i), v);
        e += v;
    };
    for (int j = first; j <= last; ++j) {
        if (m.list) {
            const int* id = m.pl.ids.data() + m.pl.start[j];
            for (int k = 0; k < m.pl.count[j]; ++k)
                if (id[k] < first || id[k] > last) term(j, id[k]);
        } else {
            for (int i = 0; i < first; ++i) term(j, i);
            for (int i = last + 1; i < m.N; ++i) term(j, i);
        }
    }
    return e;
}

// Vector::rotate(Quat) (scOOP/structures/Vector.h:162-183).
inline void quatRotate(or_vec& v, double w, double qx, double qy, double qz) {
    const double t2 = w * qx, t3 = w * qy, t4 = w * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
                 t9 = qy * qz, t10 = -qz * qz;
    const double nx = 2.0 * ((t8 + t10) * v.x + (t6 - t4) * v.y + (t3 + t7) * v.z) + v.x;
    const double ny = 2.0 * ((t4 + t6) * v.x + (t5 + t10) * v.y + (t9 - t2) * v.z) + v.y;
    const double nz = 2.0 * ((t7 - t3) * v.x + (t2 + t9) * v.y + (t5 + t8) * v.z) + v.z;
    v.x = nx; v.y = ny; v.z = nz;
}

// MoveCreator::chainMove (movecreator.cpp:305-328) with chainDisplace (:1075-1137),
// chainRotate (:1139-1256) and clusterRotate / clusterCM (:1307-1392): a random chain is
// displaced by chainmmx in a random direction or turned about its volume-weighted centre of
// (unwrapped) positions by a quaternion of half-angle up to chainr_angle, as one move.
void chainMove(or_mc& m, or_mc_stats* st) {
    if (m.chains.empty()) return;
    or_system* s = m.s;
    const or_mc_opts* o = &m.o;
    const auto ch = m.chains[(size_t)(m.rng() * m.chains.size())];
    const int first = ch.first, size = ch.second;
    std::vector<or_particle> orig(s->p + first, s->p + first + size);
    const double eold = mcChain(m, first, size, false);
    const bool displace = m.rng() < 0.5;
    if (displace) {
        or_vec dr = randomUnitSphere(m.rng);
        dr.x *= o->chainmmx / s->box[0];
        dr.y *= o->chainmmx / s->box[1];
        dr.z *= o->chainmmx / s->box[2];
        for (int j = first; j < first + size; ++j) {
            s->p[j].pos.x += dr.x; s->p[j].pos.y += dr.y; s->p[j].pos.z += dr.z;
        }
    } else {
        or_vec cm = V(0, 0, 0);
        double vol = 0.0;
        for (int j = first; j < first + size; ++j) {
            const double v = P(s, s->p[j].type, s->p[j].type).volume;
            cm.x += s->p[j].pos.x * v; cm.y += s->p[j].pos.y * v; cm.z += s->p[j].pos.z * v;
            vol += v;
        }
        cm.x /= vol; cm.y /= vol; cm.z /= vol;
        const or_vec ax = randomUnitSphere(m.rng);
        const double vc = cos(o->chainr_angle * m.rng());
        const double vs = m.rng() < 0.5 ? sqrt(1.0 - vc * vc) : -sqrt(1.0 - vc * vc);
        const double qw = vc, qx = ax.x * vs, qy = ax.y * vs, qz = ax.z * vs;
        for (int j = first; j < first + size; ++j) {
            or_particle& p = s->p[j];
            p.pos.x -= cm.x; p.pos.y -= cm.y; p.pos.z -= cm.z;
            p.pos.x *= s->box[0]; p.pos.y *= s->box[1]; p.pos.z *= s->box[2];
            quatRotate(p.pos, qw, qx, qy, qz);
            quatRotate(p.dir, qw, qx, qy, qz);
            for (int k = 0; k < 2; ++k) quatRotate(p.pd[k], qw, qx, qy, qz);
            for (int k = 0; k < 2; ++k) quatRotate(p.ch[k], qw, qx, qy, qz);
            for (int k = 0; k < 4; ++k) quatRotate(p.ps[k], qw, qx, qy, qz);
            p.pos.x /= s->box[0]; p.pos.y /= s->box[1]; p.pos.z /= s->box[2];
            p.pos.x += cm.x; p.pos.y += cm.y; p.pos.z += cm.z;
        }
    }
    const double enew = mcChain(m, first, size, true);
    const bool rej = !(enew <= eold) && !(exp(-1.0 * (enew - eold) / o->temper) > m.rng());
    if (rej) {
        std::copy(orig.begin(), orig.end(), s->p + first);
        ++st->rej_chain;
    } else {
        m.energy += enew - eold;
        if (m.matrix)
            for (const auto& c : m.chainChanges) m.em[c.first] = c.second;
        ++st->acc_chain;
    }
}

// allToAll(energyMatrix) (:502-521) into `out`, or TotalEFull::allToAll (:540-556).
double mcAllPairs(or_mc& m, std::vector<double>* out) {
    if (!out) return or_all_to_all(m.s);
    double e = 0.0;
    for (int i = 1; i < m.N; ++i) {
        const Con con = getConlist(m.s, i);
        for (int j = 0; j < i; ++j) {
            double v = pairEnergyCon(m.s, i, j, con, nullptr, nullptr);
            (*out)[emIdx(i, j)] = v;
            e += v;
        }
    }
    return e;
}

// MoveCreator::switchTypeMove (movecreator.cpp:233-303): a uniformly chosen particle with a
// switch type takes the other type of its pair, Particle::init re-derives its patch vectors,
// and moveTry(E_old, E_new + delta_mu (1 - 2 switched)) decides; a rejected switch
// re-initialises the vectors for the old type, as the reference does.  The reference draws
// the particle through ParticleVector::getSwitchPart over the molecule types; here the
// switchable particles are listed once in index order and one is drawn uniformly.
void switchMove(or_mc& m, or_mc_stats* st) {
    or_system* s = m.s;
    const or_mc_opts& o = m.o;
    const int nsw = (int)m.switchable.size();
    int k = (int)(m.rng() * nsw);
    if (k >= nsw) k = nsw - 1;
    const int t = m.switchable[k];
    const double eold = mcOld(m, t);
    const int sw = o.switched[t];
    const int pmone = 1 - 2 * sw;
    const int oldType = s->p[t].type, newType = o.switch_other[t];
    s->p[t].type = newType;
    or_particle_init(&s->p[t], &P(s, newType, newType));
    const double switchE = (double)(o.switch_dmu[t] * pmone);
    const double enew = mcTrial(m, t);
    const bool rej = !(enew + switchE <= eold) && !(exp(-1.0 * (enew + switchE - eold) / o.temper) > m.rng());
    if (rej) {
        s->p[t].type = oldType;
        or_particle_init(&s->p[t], &P(s, oldType, oldType));
        ++st->rej_switch;
    } else {
        m.energy += enew - eold;
        mcCommit(m, t);
        o.switch_other[t] = oldType;
        o.switched[t] = sw + pmone;
        ++st->acc_switch;
    }
}

// After a grand-canonical move changed N: the loop's count, the energy matrix and the pair
// list built anew (updater.cpp:166-179: initEM, genPairList); the running energy continues.
void gcResize(or_mc& m) {
    m.N = m.s->n;
    if (m.matrix) {
        const size_t sz = (size_t)m.N * (m.N > 0 ? m.N - 1 : 0) / 2 + 1;
        m.em.assign(sz, 0.0);
        m.emTrial.assign(sz, 0.0);
        mcAllPairs(m, &m.em);
    }
    if (m.list) m.pl.build(m.s, m.cut2);
}

// MoveCreator::muVTMove (movecreator.cpp:797-924) for single-particle species: a species
// drawn uniformly (getRandomMuVTType); with probability 1/2 a particle at a uniform position
// with uniform axis and patch direction (Particle::init) is inserted at the end of the
// species' block if V/(N+1) exp(chemPot - E/T) > u, else a uniformly chosen particle of the
// species is removed if N/V exp(E/T - chemPot) > u; E is the particle against every other
// with an empty conlist (mol2others), the particles behind the slot move by one.
void gcMove(or_mc& m, or_mc_stats* st) {
    or_system* s = m.s;
    const or_mc_opts& o = m.o;
    int k = (int)(m.rng() * o.n_gc);
    if (k >= o.n_gc) k = o.n_gc - 1;
    const int mt = o.gc_moltype[k];
    or_moltype* mols = const_cast<or_moltype*>(s->mols);    // the caller's records, kept current
    const int count = mols[mt].count;
    const double V = s->box[0] * s->box[1] * s->box[2];
    const Con empty;
    if (m.rng() > 0.5) {
        or_particle np;
        std::memset(&np, 0, sizeof np);
        np.pos.x = m.rng(); np.pos.y = m.rng(); np.pos.z = m.rng();
        np.dir = randomUnitSphere(m.rng);
        np.pd[0] = randomUnitSphere(m.rng);
        np.type = o.gc_type[k];
        np.molType = mt;
        or_particle_init(&np, &P(s, np.type, np.type));
        if (s->n >= o.gc_cap) { ++st->rej_insert; return; }      // no slot left (the caller sizes gc_cap)
        s->p[s->n] = np;                                          // the candidate, past the last particle
        double E = 0.0;
        for (int j = 0; j < s->n; ++j) E += pairEnergyCon(s, s->n, j, empty, nullptr, nullptr);
        if ((V / (count + 1.0)) * exp(o.gc_chempot[k] - E / o.temper) > m.rng()) {
            const int slot = mols[mt].first + count;
            std::memmove(&s->p[slot + 1], &s->p[slot], sizeof(or_particle) * (size_t)(s->n - slot));
            s->p[slot] = np;
            mols[mt].count += 1;
            for (int q = mt + 1; q < s->nmol; ++q) mols[q].first += 1;
            s->n += 1;
            m.energy += E;
            ++st->acc_insert;
            gcResize(m);
        } else {
            ++st->rej_insert;
        }
    } else {
        if (count == 0) { ++st->rej_delete; return; }
        int t = mols[mt].first + (int)(m.rng() * count);
        if (t >= mols[mt].first + count) t = mols[mt].first + count - 1;
        double E = 0.0;
        for (int j = 0; j < s->n; ++j)
            if (j != t) E += pairEnergyCon(s, t, j, empty, nullptr, nullptr);
        if (((double)count / V) * exp(E / o.temper - o.gc_chempot[k]) > m.rng()) {
            std::memmove(&s->p[t], &s->p[t + 1], sizeof(or_particle) * (size_t)(s->n - t - 1));
            mols[mt].count -= 1;
            for (int q = mt + 1; q < s->nmol; ++q) mols[q].first -= 1;
            s->n -= 1;
            m.energy -= E;
            ++st->acc_delete;
            gcResize(m);
        } else {
            ++st->rej_delete;
        }
    }
}

}  // namespace

extern "C" or_mc* or_mc_open(or_system* s, const or_mc_opts* o) {
    const bool gc = o && o->grand_every > 0 && o->n_gc > 0 && o->gc_moltype && o->gc_type && o->gc_chempot;
    if (!s || !o || (s->n <= 0 && !gc)) return nullptr;
    if (gc && o->switchprob > 0.0) return nullptr;             // not combined with switching here
    if (o->shave > 0.0 && (o->ptype < 0 || o->ptype > 5)) return nullptr;     // couplings 0..5
    auto t0 = std::chrono::steady_clock::now();
    or_mc* m = new or_mc();
    m->s = s;
    m->o = *o;
    m->rng = Rng{(uint64_t)o->seed * 0x2545F4914F6CDD1Dull + 1};
    m->N = s->n;
    m->shprob = s->n > 0 ? o->shave / (double)s->n : 0.0;
    m->gc = gc;
    m->matrix = o->energy_matrix != 0;
    if (o->pairlist_update > 0) {
        // the pair-list cutoff of main.cpp:117-126 (equal step sizes: AVER is the step)
        double c = o->transmx;
        c *= (1 + o->pairlist_update) * 2;
        c += sqrt(s->sqmaxcut);
        m->cut2 = c * c;
        m->list = true;
    }
    if (m->matrix) {
        size_t sz = (size_t)m->N * (m->N - 1) / 2 + 1;
        m->em.assign(sz, 0.0);
        m->emTrial.assign(sz, 0.0);
        m->energy = mcAllPairs(*m, &m->em);      // initEM
    } else {
        m->energy = or_all_to_all(s);
    }
    if (m->list) m->pl.build(s, m->cut2);          // before the first sweep (updater.cpp:176-190)
    if (o->chainprob > 0.0) buildChains(*m);
    if (o->switchprob > 0.0 && o->switch_other && o->switch_dmu && o->switched) {
        for (int i = 0; i < s->n; ++i)
            if (o->switch_other[i] >= 0) m->switchable.push_back(i);
        // no switchable particle: no switch moves (initSwitchList, inicializer.cpp:77-81)
        if (!m->switchable.empty()) m->swprob = o->switchprob;
    }
    m->setupSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return m;
}

extern "C" void or_mc_close(or_mc* m) { delete m; }

extern "C" double or_mc_energy(const or_mc* m) { return m ? m->energy : 0.0; }

extern "C" double or_mc_setup_seconds(const or_mc* m) { return m ? m->setupSeconds : 0.0; }

// Runs `moves` more steps of the sweep loop (updater.cpp:192-230); stats accumulate into st
// (moves, acceptance counts, running energy, seconds spent here).
extern "C" int or_mc_advance(or_mc* m, long moves, or_mc_stats* st) {
    if (!m || !st || moves < 0) return -1;
    or_system* s = m->s;
    const or_mc_opts* o = &m->o;
    auto t0 = std::chrono::steady_clock::now();
    // the end of a sweep: its grand-canonical move when one is due (updater.cpp:164-179)
    auto endSweep = [&]() {
        if (m->gc && m->sweep % o->grand_every == 0) gcMove(*m, st);
        m->step = 1;
        ++m->sweep;
    };
    long done = 0;
    while (done < moves) {
        if (m->N == 0) {                    // an empty box: a sweep of no steps, counted as one
            ++done;
            endSweep();
            continue;
        }
        if (m->step > m->N) {
            endSweep();
            if (m->N == 0) continue;        // its grand-canonical move emptied the box
        }
        if (m->step == 1 && m->list && m->sweep > 1 && m->sweep % o->pairlist_update == 0) m->pl.build(s, m->cut2);
        ++m->step;
        ++done;
        const int N = m->N;
        double u = m->rng();
        if (u < m->shprob) {
            // pressureMove (movecreator.cpp:330-546), every coupling; a box with an edge that is
            // not positive is rejected before its energy is evaluated
            BoxTrial bt;
            double enermove = bt.propose(s->box, o, N, m->rng);
            bool rej = !(s->box[0] > 0.0 && s->box[1] > 0.0 && s->box[2] > 0.0);
            double enew = 0.0;
            if (!rej) {
                enew = mcAllPairs(*m, m->matrix ? &m->emTrial : nullptr);
                enermove += enew;
                rej = !(enermove <= m->energy) && !(exp(-1.0 * (enermove - m->energy) / o->temper) > m->rng());
            }
            if (rej) { bt.reject(s->box); ++st->rej_vol; }
            else {
                ++st->acc_vol;
                m->energy = enew;
                if (m->matrix) std::swap(m->em, m->emTrial);   // update(): swapEMatrices
            }
            continue;
        }
        if (u < m->shprob + m->o.chainprob) {  // updater.cpp:215-218
            chainMove(*m, st);
            continue;
        }
        if (u < m->shprob + m->o.chainprob + m->swprob) {      // updater.cpp:219-222
            switchMove(*m, st);
            continue;
        }
        int target = (int)(m->rng() * N);
        or_particle orig = s->p[target];
        const or_param& d = P(s, orig.type, orig.type);
        bool displace = (m->rng() < 0.5) || d.geotype[0] >= SP;
        double eold = mcOld(*m, target);
        if (displace) {
            or_vec dr = randomUnitSphere(m->rng);
            s->p[target].pos.x += dr.x * o->transmx / s->box[0];
            s->p[target].pos.y += dr.y * o->transmx / s->box[1];
            s->p[target].pos.z += dr.z * o->transmx / s->box[2];
        } else {
            double ang = o->rot_angle * m->rng();
            or_vec ax = randomUnitSphere(m->rng);
            or_psc_rotate(&s->p[target], d.geotype[0], ang, ax, m->rng() < 0.5);
            ortho(s->p[target].pd[0], s->p[target].dir);
        }
        double enew = mcTrial(*m, target);
        bool rej = !(enew <= eold) && !(exp(-1.0 * (enew - eold) / o->temper) > m->rng());
        if (rej) {
            s->p[target] = orig;
            if (displace) ++st->rej_trans; else ++st->rej_rot;
        } else {
            m->energy += enew - eold;
            mcCommit(*m, target);
            if (displace) ++st->acc_trans; else ++st->acc_rot;
        }
    }
    if (m->N > 0 && m->step > m->N) endSweep();  // the block ended on a sweep's last step
    st->moves += done;
    st->energy = m->energy;
    st->seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

// Runs whole sweeps: the steps left in the current sweep, then full sweeps of the particle
// count each has at its start (grand-canonical moves change it between sweeps).
extern "C" int or_mc_sweeps(or_mc* m, long sweeps, or_mc_stats* st) {
    if (!m || !st || sweeps < 0) return -1;
    const long target = m->sweep + sweeps;
    while (m->sweep < target) {
        const long left = m->N > 0 ? m->N - m->step + 1 : 1;
        if (or_mc_advance(m, left, st) != 0) return -1;
    }
    return 0;
}

extern "C" int or_mc_run(or_system* s, const or_mc_opts* o, or_mc_stats* st) {
    std::memset(st, 0, sizeof(*st));
    or_mc* m = or_mc_open(s, o);
    if (!m) return -1;
    st->energy_start = m->energy;
    long total = o->nsweeps * (long)s->n;
    if (o->max_moves > 0 && o->max_moves < total) total = o->max_moves;
    int rc = m->gc ? or_mc_sweeps(m, o->nsweeps, st) : or_mc_advance(m, total, st);
    st->seconds += m->setupSeconds;
    or_mc_close(m);
    return rc;
}

// ---- Wang-Landau order parameters --------------------------------------------------------
namespace {

// Order 7 (WangLandau::particlesInContact / contParticlesAll, scOOP/mc/wanglandau.h:603-676):
// a particle is in contact with particle 0 when its minimum-image distance squared is below
// WL_CONTACTS = 36 (scOOP/structures/macros.h:107); the count runs over particles 1..N-1 of
// type wlmtype, the bin is ceil((count - minorder) / dorder) (contParticlesOrder).
bool wlInContact(const or_system* s, const or_vec& a, const or_vec& p0) {
    double x = a.x - p0.x, y = a.y - p0.y, z = a.z - p0.z;
    x = s->box[0] * (x - anint(x));
    y = s->box[1] * (y - anint(y));
    z = s->box[2] * (z - anint(z));
    return x * x + y * y + z * z < 36.0;
}

long wlContactsAll(const or_system* s, int wlmtype) {
    long c = 0;
    for (int i = 1; i < s->n; ++i)
        if (s->p[i].type == wlmtype && wlInContact(s, s->p[i].pos, s->p[0].pos)) ++c;
    return c;
}

long wlContactBin(long count, double minorder, double dorder) {
    return (long)std::ceil(((double)count - minorder) / dorder);
}

// Order 2 (Mesh, scOOP/mc/mesh.cpp; WangLandau::meshOrderMoveMolecule, wanglandau.cpp:7-47):
// an xy mesh of squares sigma(wlmtype) / 3 wide; every particle of type wlmtype occupies
// the 3 x 3 squares around the one holding it (each occupation counts down from 0); the
// order is the size of the largest 4-connected periodic cluster of free squares
// (findHoles), binned as (long)((size - minorder) / dorder).
double wlInbox(double a) {          // INBOX (macros.h:119)
    double ip;
    return a > 0 ? std::modf(a, &ip) : std::modf(a, &ip) + 1;
}

struct WlMesh {
    int dim[2] = {0, 0};
    std::vector<int> data, tmp;

    int square(int x, int y) const { return x + dim[0] * y; }
    void squares(int x, int y, int sq[9]) const {       // Mesh::meshSquare
        const int xm = x - 1 < 0 ? dim[0] - 1 : x - 1, xp = x + 1 == dim[0] ? 0 : x + 1;
        const int ym = y - 1 < 0 ? dim[1] - 1 : y - 1, yp = y + 1 == dim[1] ? 0 : y + 1;
        sq[0] = square(x, y); sq[1] = square(xm, y); sq[2] = square(xp, y);
        sq[3] = square(x, ym); sq[4] = square(xm, ym); sq[5] = square(xp, ym);
        sq[6] = square(x, yp); sq[7] = square(xm, yp); sq[8] = square(xp, yp);
    }
    int cellX(double x) const { return (int)(wlInbox(x) * dim[0]); }
    int cellY(double y) const { return (int)(wlInbox(y) * dim[1]); }
    bool valid(int q) const { return q >= 0 && q < dim[0] * dim[1]; }
    // Mesh::addPart: 1 when every square was occupied already (no hole shrank)
    int add(double x, double y) {
        int sq[9], onhole = 1;
        squares(cellX(x), cellY(y), sq);
        for (int i = 0; i < 9; ++i) {
            if (!valid(sq[i])) continue;        // the reference reports these and writes anyway
            if (data[sq[i]] >= 0) onhole = 0;
            data[sq[i]]--;
        }
        return onhole;
    }
    // Mesh::removePart: 0 at the first square it frees (the rest are left as they are)
    int remove(double x, double y) {
        int sq[9];
        squares(cellX(x), cellY(y), sq);
        for (int i = 0; i < 9; ++i) {
            if (!valid(sq[i])) continue;
            data[sq[i]]++;
            if (data[sq[i]] == 0) return 0;
        }
        return 1;
    }
    void fill(const or_system* s, int wlmtype) {       // Mesh::meshFill
        std::fill(data.begin(), data.end(), 0);
        for (int i = 0; i < s->n; ++i)
            if (s->p[i].type == wlmtype) add(s->p[i].pos.x, s->p[i].pos.y);
    }
    int findHoles() {                                   // Mesh::findHoles
        const int L = dim[0] * dim[1];
        int n = 0, maxsize = 0;
        for (int i = 0; i < L; ++i) {
            tmp[i] = 0;
            if (data[i] > 0) data[i] = 0;
        }
        for (int i = 0; i < L;) {
            if (data[i] != 0) { ++i; continue; }
            ++n;
            data[i] = n;
            int size = 1, li = 0;
            tmp[0] = i;
            while (li < size) {
                const int j = tmp[li], x = j % dim[0], y = j / dim[0];
                const int nb[4] = {square(x - 1 < 0 ? dim[0] - 1 : x - 1, y), square(x + 1 == dim[0] ? 0 : x + 1, y),
                                   square(x, y - 1 < 0 ? dim[1] - 1 : y - 1), square(x, y + 1 == dim[1] ? 0 : y + 1)};
                for (int k = 0; k < 4; ++k)
                    if (data[nb[k]] == 0) {
                        data[nb[k]] = n;
                        tmp[size++] = nb[k];
                    }
                ++li;
            }
            if (size > maxsize) maxsize = size;
        }
        return maxsize;
    }
    // Mesh::meshInit with the box now: -1 when the mesh has no square
    int init(const or_system* s, int wlmtype) {
        if (wlmtype < 0 || wlmtype >= OR_MAXT) return -1;
        const double ms = s->params[wlmtype * OR_MAXT + wlmtype].sigma / 3.0;
        if (!(ms > 0.0)) return -1;
        dim[0] = (int)(s->box[0] / ms);
        dim[1] = (int)(s->box[1] / ms);
        if (dim[0] < 1 || dim[1] < 1) return -1;
        data.assign((size_t)dim[0] * dim[1], 0);
        tmp.assign((size_t)dim[0] * dim[1] + 1, 0);
        fill(s, wlmtype);
        return findHoles();
    }
};

long wlMeshBin(int size, double minorder, double dorder) { return (long)(((double)size - minorder) / dorder); }

}  // namespace

// WangLandau::init (scOOP/mc/wanglandau.cpp:49-137): the starting bin of each order
// parameter.  Order 1: Conf::massCenter (scOOP/structures/Conf.cpp:78-95) over the
// anInt-wrapped positions weighted by the Ia_param volumes, then zOrder
// (wanglandau.h:551-554); 2: the mesh hole (above); 3: zOrient (:321-324, floor); 4:
// twoPartDist (:395-398); 7: the contacts (above); 8 / 9: the box lengths (:375-382).
// Returns -1 for another order parameter (5 and 6, the pore orders, end the reference's
// own init with a null-pointer write: radiusholeAll, wanglandau.cpp:306-318, never
// allocates its histogram) or a mesh without squares.
extern "C" int or_wl_orders(const or_system* s, const int wlm[2], int wlmtype, const double minorder[2],
                            const double dorder[2], long out[2], double syscm[3], double* sysvolume) {
    double sv = 0.0;
    for (int i = 0; i < s->n; ++i) sv += s->params[s->p[i].type * OR_MAXT + s->p[i].type].volume;
    or_vec cm = V(0, 0, 0);
    for (int i = 0; i < s->n; ++i) {
        const double v = s->params[s->p[i].type * OR_MAXT + s->p[i].type].volume;
        const or_vec& r = s->p[i].pos;
        cm.x += (r.x - anint(r.x)) * v;
        cm.y += (r.y - anint(r.y)) * v;
        cm.z += (r.z - anint(r.z)) * v;
    }
    cm.x /= sv; cm.y /= sv; cm.z /= sv;
    syscm[0] = cm.x; syscm[1] = cm.y; syscm[2] = cm.z;
    *sysvolume = sv;
    out[0] = out[1] = 0;
    for (int k = 0; k < 2; ++k) {
        if (wlm[k] == 0) continue;
        switch (wlm[k]) {
        case 1: out[k] = (long)std::ceil(((s->p[0].pos.z - cm.z) * s->box[2] - minorder[k]) / dorder[k]); break;
        case 3: out[k] = (long)std::floor((s->p[0].dir.z - minorder[k]) / dorder[k]); break;
        case 4: {
            or_vec r = image(s->p[0].pos, s->p[1].pos, s->box);
            out[k] = (long)std::ceil((std::sqrt(r.x * r.x + r.y * r.y) - minorder[k]) / dorder[k]);
            break;
        }
        case 2: {
            WlMesh m;
            const int size = m.init(s, wlmtype);
            if (size < 0) return -1;
            out[k] = wlMeshBin(size, minorder[k], dorder[k]);
            break;
        }
        case 7: out[k] = wlContactBin(wlContactsAll(s, wlmtype), minorder[k], dorder[k]); break;
        case 8: out[k] = (long)std::ceil((s->box[0] - minorder[k]) / dorder[k]); break;
        case 9: out[k] = (long)std::ceil((s->box[1] - minorder[k]) / dorder[k]); break;
        default: return -1;
        }
    }
    return 0;
}

// ---- Wang-Landau move loop ------------------------------------------------------------------
// The reference's sequential loop with a Wang-Landau bias, single-particle and volume moves:
// MoveCreator::partDisplace / partRotate with WangLandau::run / runRot (movecreator.cpp:
// 947-1028, wanglandau.h:124-217): the bins after the move (order 1: the system centre moves
// by volume * displacement / sysvolume, zDir :293-299; 3: zOrient of particle 0; 4:
// twoPartDist; 7: the contact count, recounted when particle 0 moves, else changed by the
// moved particle's old and new contact (contParticlesMoveMolecule, :516-532); 2: the mesh,
// updated by Mesh::addPart / removePart and refilled when a hole may have changed
// (meshOrderMoveMolecule), restored on rejection), a bin outside the histogram rejects the move, else
// moveTry(energy + w[new] - w[cur], enermove); then accept / reject (:262-290): the current
// bin's weight drops by alpha and its count grows by one.  Every 1000 sweeps
// WangLandau::update (:66-120, integer max / min) halves alpha when the histogram is flat;
// below WL_ALPHATOL the run stops.
extern "C" int or_wl_run(or_system* s, const or_mc_opts* o, or_wl* wl, or_mc_stats* st) {
    std::memset(st, 0, sizeof(*st));
    Rng rng{(uint64_t)o->seed * 0x2545F4914F6CDD1Dull + 1};
    const int N = s->n;
    if (N <= 0) return -1;
    const int dim = wl->wlm[1] > 0 ? 2 : 1;
    const long nb = (long)wl->len[0] * wl->len[1];
    double sv = 0.0;
    for (int i = 0; i < N; ++i) sv += P(s, s->p[i].type, s->p[i].type).volume;
    or_vec cm = V(0, 0, 0);
    for (int i = 0; i < N; ++i) {
        const double v = P(s, s->p[i].type, s->p[i].type).volume;
        const or_vec& r = s->p[i].pos;
        cm.x += (r.x - anint(r.x)) * v; cm.y += (r.y - anint(r.y)) * v; cm.z += (r.z - anint(r.z)) * v;
    }
    cm.x /= sv; cm.y /= sv; cm.z /= sv;
    bool uses[10] = {};
    for (int k = 0; k < dim; ++k) {
        if (wl->wlm[k] < 1 || wl->wlm[k] > 9 || wl->wlm[k] == 5 || wl->wlm[k] == 6) return -3;
        uses[wl->wlm[k]] = true;
    }
    const int wlmtype = wl->wlmtype;
    long contacts = uses[7] ? wlContactsAll(s, wlmtype) : 0;
    WlMesh mesh, origmesh;
    if (uses[2] && mesh.init(s, wlmtype) < 0) return -3;
    auto idx = [&](const long* b) { return b[0] + b[1] * (long)wl->len[0]; };
    auto inRange = [&](const long* b) {
        for (int k = 0; k < dim; ++k)
            if (b[k] < 0 || b[k] >= wl->len[k]) return false;
        return true;
    };
    auto visit = [&]() {
        wl->weights[idx(wl->cur)] -= wl->alpha;
        wl->hist[idx(wl->cur)] += 1;
    };
    const double shprob = o->shave / (double)N;
    if (shprob > 0.0 && (o->ptype < 0 || o->ptype > 5)) return -2;
    // MoveCreator::pressureMove (movecreator.cpp:330-546) with WangLandau::runPress
    // (wanglandau.h:168-196): the bins of the trial box (order 1 keeps the centre, and ptype
    // 2 keeps order 1; 4 the two particles' distance; 8 / 9 the box lengths)
    auto volumeMove = [&]() {
        const double energy = or_all_to_all(s);
        BoxTrial bt;
        double enermove = bt.propose(s->box, o, N, rng);
        long nw[2] = {wl->cur[0], wl->cur[1]};
        long cntNew = contacts;
        if (uses[2]) origmesh = mesh;
        for (int k = 0; k < dim; ++k) {
            switch (wl->wlm[k]) {
            case 2: nw[k] = wlMeshBin(mesh.init(s, wlmtype), wl->minorder[k], wl->dorder[k]); break;
            case 7:
                cntNew = wlContactsAll(s, wlmtype);
                nw[k] = wlContactBin(cntNew, wl->minorder[k], wl->dorder[k]);
                break;
            case 1:
                if (o->ptype != 2)
                    nw[k] = (long)std::ceil(((s->p[0].pos.z - cm.z) * s->box[2] - wl->minorder[k]) / wl->dorder[k]);
                break;
            case 4: {
                or_vec r = image(s->p[0].pos, s->p[1].pos, s->box);
                nw[k] = (long)std::ceil((std::sqrt(r.x * r.x + r.y * r.y) - wl->minorder[k]) / wl->dorder[k]);
                break;
            }
            case 8: nw[k] = (long)std::ceil((s->box[0] - wl->minorder[k]) / wl->dorder[k]); break;
            case 9: nw[k] = (long)std::ceil((s->box[1] - wl->minorder[k]) / wl->dorder[k]); break;
            default: break;
            }
        }
        bool rej = !inRange(nw) || !(s->box[0] > 0 && s->box[1] > 0 && s->box[2] > 0);
        if (!rej) {
            enermove += or_all_to_all(s);
            const double eo = energy + wl->weights[idx(nw)] - wl->weights[idx(wl->cur)];
            rej = !(enermove <= eo) && !(exp(-1.0 * (enermove - eo) / o->temper) > rng());
        }
        if (rej) {
            bt.reject(s->box);
            if (uses[2]) mesh = origmesh;
            ++st->rej_vol;
        } else {
            wl->cur[0] = nw[0]; wl->cur[1] = nw[1];
            contacts = cntNew;
            ++st->acc_vol;
        }
        visit();
    };
    auto t0 = std::chrono::steady_clock::now();
    long moves = 0;
    for (long sweep = 1; sweep <= o->nsweeps; ++sweep) {
        for (int step = 1; step <= N; ++step) {
            if (o->max_moves > 0 && moves >= o->max_moves) goto finish;
            ++moves;
            if (shprob > 0.0 && rng() < shprob) {      // Updater::simulate's step choice
                volumeMove();
                continue;
            }
            int target = (int)(rng() * N);
            or_particle orig = s->p[target];
            const or_param& d = P(s, orig.type, orig.type);
            const or_vec cmOld = cm;
            double eold = or_one_to_all(s, target);
            bool displace = (rng() < 0.5) || d.geotype[0] >= SP;
            long nw[2] = {wl->cur[0], wl->cur[1]};
            long cntNew = contacts;
            if (uses[2]) origmesh = mesh;
            if (displace) {
                or_vec dr = randomUnitSphere(rng);
                dr.x *= o->transmx / s->box[0]; dr.y *= o->transmx / s->box[1]; dr.z *= o->transmx / s->box[2];
                s->p[target].pos.x += dr.x; s->p[target].pos.y += dr.y; s->p[target].pos.z += dr.z;
                for (int k = 0; k < dim; ++k) {
                    if (wl->wlm[k] == 1) {
                        cm.x += dr.x * d.volume / sv; cm.y += dr.y * d.volume / sv; cm.z += dr.z * d.volume / sv;
                        nw[k] = (long)std::ceil(((s->p[0].pos.z - cm.z) * s->box[2] - wl->minorder[k]) / wl->dorder[k]);
                    } else if (wl->wlm[k] == 4) {
                        or_vec r = image(s->p[0].pos, s->p[1].pos, s->box);
                        nw[k] = (long)std::ceil((std::sqrt(r.x * r.x + r.y * r.y) - wl->minorder[k]) / wl->dorder[k]);
                    } else if (wl->wlm[k] == 7) {
                        if (target == 0) {
                            cntNew = wlContactsAll(s, wlmtype);
                        } else if (orig.type == wlmtype) {
                            cntNew += wlInContact(s, s->p[target].pos, s->p[0].pos) ? 1 : 0;
                            cntNew -= wlInContact(s, orig.pos, s->p[0].pos) ? 1 : 0;
                        }
                        nw[k] = wlContactBin(cntNew, wl->minorder[k], wl->dorder[k]);
                    } else if (wl->wlm[k] == 2 && orig.type == wlmtype) {
                        const or_vec& np = s->p[target].pos;
                        if (mesh.cellX(np.x) != mesh.cellX(orig.pos.x) || mesh.cellY(np.y) != mesh.cellY(orig.pos.y)) {
                            int change = mesh.add(np.x, np.y);
                            if (change) change = mesh.remove(orig.pos.x, orig.pos.y);
                            if (!change) {
                                mesh.fill(s, wlmtype);
                                nw[k] = wlMeshBin(mesh.findHoles(), wl->minorder[k], wl->dorder[k]);
                            }
                        }
                    }
                }
            } else {
                double ang = o->rot_angle * rng();
                or_vec ax = randomUnitSphere(rng);
                or_psc_rotate(&s->p[target], d.geotype[0], ang, ax, rng() < 0.5);
                ortho(s->p[target].pd[0], s->p[target].dir);
                for (int k = 0; k < dim; ++k)
                    if (wl->wlm[k] == 3 && target == 0)
                        nw[k] = (long)std::floor((s->p[0].dir.z - wl->minorder[k]) / wl->dorder[k]);
            }
            bool rej = !inRange(nw);
            double wlener = 0.0, enew = 0.0;
            if (!rej) {
                wlener = wl->weights[idx(nw)] - wl->weights[idx(wl->cur)];
                enew = or_one_to_all(s, target);
                double eo = eold + wlener;
                rej = !(enew <= eo) && !(exp(-1.0 * (enew - eo) / o->temper) > rng());
            }
            if (rej) {
                s->p[target] = orig;
                cm = cmOld;
                if (uses[2]) mesh = origmesh;
                if (displace) ++st->rej_trans; else ++st->rej_rot;
            } else {
                wl->cur[0] = nw[0]; wl->cur[1] = nw[1];
                contacts = cntNew;
                st->energy += enew - eold;
                if (displace) ++st->acc_trans; else ++st->acc_rot;
            }
            visit();
        }
        if (wl->alpha > 0.0 && sweep % 1000 == 0) {
            long mn = wl->hist[0], mx = wl->hist[0];
            for (long i = 0; i < nb; ++i) { mn = std::min(mn, wl->hist[i]); mx = std::max(mx, wl->hist[i]); }
            if (mn > 1000 && o->temper * std::log((double)(mx / mn)) < 0.0001) {
                if (wl->alpha < 1.0e-8) { wl->converged = 1; break; }
                wl->alpha /= 2.0;
                wl->updates += 1;
                const double wmin = wl->weights[0];
                for (long i = 0; i < nb; ++i) { wl->hist[i] = 0; wl->weights[i] -= wmin; }
            }
        }
    }
finish:
    st->moves = moves;
    st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}
