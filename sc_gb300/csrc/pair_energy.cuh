// pair_energy.cuh -- FP64 pair energy of patchy spherocylinders and spheres on sm_103a.
//
// Device implementation of the reference's PairE (scOOP/mc/paire.h:1202-1228) and
// the functors it dispatches to.  Every arithmetic expression keeps the
// reference's operand order and the translation units are compiled with
// --fmad=false, so that overlap / cutoff / intersection verdicts are bit-identical
// to the reference's on the same inputs; transcendental calls (pow, cos, acos)
// may differ by a few ulp, which the 1e-12 relative energy tolerance absorbs.
//
// Data layout (structure of arrays in HBM):
//   pos[i]   double4  x, y, z in box fractions (never re-wrapped), w = compact type index
//   dir[i]   double4  unit axis, w unused
//   patch[i] PatchSet patchdir[2], patchsides[4], chdir[2]   (192 B)
//   mol[i]   int4     molecule type, position inside the molecule, molecule size, unused
#pragma once

#include <cuda_runtime.h>

#include "sc_common.h"

namespace scg {

struct DevCtx {
    const PairParam* params;   // ntypes x ntypes, row-major [compact t1][compact t2]
    const MolParam* mols;      // per molecule type
    int ntypes;
    int n;
    double sqmaxcut;
};

// What the pair energy reads of one particle.
struct PView {
    double3 pos;
    double3 dir;
    const PatchSet* patch;
    int type;       // compact type index
    int index;      // particle index (bond partner identity)
    int molType;
};

// ConList of particle 1 (ParticleVector::getConlist, scOOP/structures/Conf.h:90-147).
struct Con {
    int idx[4];     // tail, head, second tail, second head; -1 = none
    int isEmpty;
    const MolParam* m;
};

__device__ __forceinline__ double3 mk(double x, double y, double z) { return make_double3(x, y, z); }
__device__ __forceinline__ double dot3(const double3& a, const double3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 ld3(const double (&v)[3]) { return mk(v[0], v[1], v[2]); }
__device__ __forceinline__ double3 scl(double s, const double3& v) { return mk(v.x * s, v.y * s, v.z * s); }
__device__ __forceinline__ double3 neg3(const double3& v) { return mk(-1.0 * v.x, -1.0 * v.y, -1.0 * v.z); }
__device__ __forceinline__ double vlen(const double3& v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ double3 cross3(const double3& A, const double3& B) {
    return mk(A.y * B.z - A.z * B.y, -A.x * B.z + A.z * B.x, A.x * B.y - A.y * B.x);
}
__device__ __forceinline__ double3 perpProj(const double3& a, const double3& B) {
    double dp = dot3(a, B);
    return mk(a.x - B.x * dp, a.y - B.y * dp, a.z - B.z * dp);
}
__device__ __forceinline__ void normalise3(double3& v) {
    double t = vlen(v);
    if (t != 0.0) { t = 1.0 / t; v.x *= t; v.y *= t; v.z *= t; }
}

// Minimum image in box fractions, scaled to real space (Cuboid::image, geometry.h:110-128).
// rint() is the round-half-even the reference obtains from the 1.5*2^52 trick.
__device__ __forceinline__ double3 imageVec(const double3& r1, const double3& r2, const double3& box) {
    double dx = r1.x - r2.x, dy = r1.y - r2.y, dz = r1.z - r2.z;
    return mk(box.x * (dx - rint(dx)), box.y * (dy - rint(dy)), box.z * (dz - rint(dz)));
}

__device__ __forceinline__ double harmonicE(double a, double eq, double k) { return k * (a - eq) * (a - eq) * 0.5; }

__device__ __forceinline__ double fanglScale(double a, double pcangl, double pcanglsw) {
    if (a <= pcanglsw) return 0.0;
    return (a >= pcangl) ? 1.0 : (0.5 - ((pcanglsw + pcangl) * 0.5 - a) / (pcangl - pcanglsw));
}

// Closest vector between two segments (EPatch::minDistSegments, scOOP/mc/paire.cpp:85-241).
static __device__ __noinline__ double3 minDistSegments(double3 segA, double3 segB, double halfl1, double halfl2, double3 r_cm) {
    double3 u = scl(2.0 * halfl1, segA), v = scl(2.0 * halfl2, segB), w;
    w.x = segB.x * halfl2 - segA.x * halfl1 - r_cm.x;
    w.y = segB.y * halfl2 - segA.y * halfl1 - r_cm.y;
    w.z = segB.z * halfl2 - segA.z * halfl1 - r_cm.z;
    double a = dot3(u, u), b = dot3(u, v), c = dot3(v, v), d = dot3(u, w), e = dot3(v, w);
    double D = a * c - b * b;
    double sc, sN = D, sD = D, tc, tN = D, tD = D;
    bool par = false;
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
    double3 vec = mk(u.x * sc + w.x - v.x * tc, u.y * sc + w.y - v.y * tc, u.z * sc + w.z - v.z * tc);
    if (par) {
        // parallel segments: also test from the other segment's end (paire.cpp:170-238)
        w.x = segA.x * halfl1 - segB.x * halfl2 + r_cm.x;
        w.y = segA.y * halfl1 - segB.y * halfl2 + r_cm.y;
        w.z = segA.z * halfl1 - segB.z * halfl2 + r_cm.z;
        d = dot3(v, w);
        e = dot3(u, w);
        D = a * c - b * b;
        sN = D; sD = D; tN = D; tD = D;
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
        double3 vec2 = mk(v.x * sc + w.x - u.x * tc, v.y * sc + w.y - u.y * tc, v.z * sc + w.z - u.z * tc);
        if (dot3(vec2, vec2) < dot3(vec, vec)) return vec2;
    }
    return vec;
}

struct PatchV { double3 dir, s0, s1; };

// --- intersections of a segment with the attractive wedge of a patch (paire.h:86-181, 499-827)

__device__ __forceinline__ void testIntrPatch(const double3& dir, const double3& patchdir, double3 vec, double cospatch,
                                              double ti, double* in) {
    vec = perpProj(vec, dir);
    if (dot3(patchdir, vec) >= cospatch * vlen(vec)) {
        if (in[0] == 0) { in[0] = ti; return; }
        if (in[1] == 0 && in[0] != ti) { in[1] = ti; return; }
    }
}

__device__ __forceinline__ void scToInfiIntr(const double3& d1, const double3& d2, const PatchV& P, const double3& r_cm,
                                             double pcanglsw, double halfl1, double halfl2, double* in, double x1) {
    if ((x1 >= halfl2) || (x1 <= -halfl2)) return;
    double3 v1 = mk(d2.x * x1 - r_cm.x, d2.y * x1 - r_cm.y, d2.z * x1 - r_cm.z);
    double e = dot3(d1, v1);
    if ((e >= halfl1) || (e <= -halfl1)) return;
    testIntrPatch(d1, P.dir, v1, pcanglsw, x1, in);
}

__device__ __forceinline__ void testIntrAtC(const double3& d1, const double3& d2, const PatchV& P, const double3& r_cm,
                                            double pcanglsw, double rcutSq, double halfl1, double halfl2, double* in) {
    double3 v1 = cross3(neg3(r_cm), d1), v2 = cross3(d2, d1);
    double a = dot3(v2, v2), b = 2 * dot3(v1, v2), c = -rcutSq + dot3(v1, v1), d = b * b - 4 * a * c;
    if (d >= 0) {
        d = sqrt(d);
        a = 0.5 / a;
        scToInfiIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, (-b + d) * a);
        if (d > 0) scToInfiIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, (-b - d) * a);
    }
}

__device__ __forceinline__ bool planeIntersect(const double3& dirA, const double3& dirB, double halfl, const double3& r_cm,
                                               const double3& w_vec, double cospatch, double& ti, double& c, double& d) {
    double3 nplane = cross3(dirA, w_vec);
    double a = dot3(nplane, dirB);
    c = 1.0; d = 1.0;
    if (a == 0.0) return false;
    ti = dot3(nplane, r_cm) / a;
    if ((ti > halfl) || (ti < -halfl)) return false;
    double3 dv = mk(ti * dirB.x - r_cm.x, ti * dirB.y - r_cm.y, ti * dirB.z - r_cm.z);
    c = dot3(dv, w_vec);
    if (c * cospatch < 0) return false;
    d = fabs(dot3(dv, dirA)) - halfl;
    return true;
}

__device__ __forceinline__ void scToEndSpIntr(const double3& d1, const double3& d2, const PatchV& P, const double3& r_cm,
                                              double pcanglsw, double halfl1, double halfl2, double* in, double x1) {
    if ((x1 >= halfl2) || (x1 <= -halfl2)) return;
    double3 v1 = mk(d2.x * x1 - r_cm.x, d2.y * x1 - r_cm.y, d2.z * x1 - r_cm.z);
    double e = dot3(d1, v1);
    if ((e >= halfl1) || (e <= -halfl1)) testIntrPatch(d1, P.dir, v1, pcanglsw, x1, in);
}

__device__ __forceinline__ void capSphereIntersections(const double3& d1, const double3& d2, const PatchV& P,
                                                       const double3& r_cm, double* in, double pcanglsw, double halfl1,
                                                       double halfl2, double b, double c) {
    double d = b * b - 4 * c;
    if (d >= 0) {
        d = sqrt(d);
        scToEndSpIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, (-b + d) * 0.5);
        if (d > 0) scToEndSpIntr(d1, d2, P, r_cm, pcanglsw, halfl1, halfl2, in, (-b - d) * 0.5);
    }
}

__device__ __forceinline__ void endInsideTest(const double3& d1, const double3& d2, const PatchV& P, const double3& r_cm,
                                              double pcanglsw, double rcutSq, double halfl1, double halfl2, double* in) {
    double3 v1 = mk(d2.x * halfl2 - r_cm.x, d2.y * halfl2 - r_cm.y, d2.z * halfl2 - r_cm.z);
    double a = dot3(v1, d1);
    double3 v2 = mk(v1.x - d1.x * a, v1.y - d1.y * a, v1.z - d1.z * a);
    double b = dot3(v2, v2), d = fabs(a) - halfl1;
    double c = (d <= 0) ? b : d * d + b;
    if (c < rcutSq) testIntrPatch(d1, P.dir, v1, pcanglsw, halfl2, in);
}

// Psc::pscIntersect (paire.h:499-583): 2 if segment 2 crosses the wedge of patch 1 twice.
static __device__ __noinline__ int pscIntersect(double3 d1, double3 d2, PatchV P, double3 r_cm, double* io,
                                         double pcanglsw, double rcutSq, double halfl1, double halfl2) {
    double c, d, ti, disti;
    double in[2] = {0, 0};
    if (planeIntersect(d1, d2, halfl2, r_cm, P.s0, pcanglsw, ti, c, d)) {
        disti = (d <= 0) ? c * c : d * d + c * c;
        if (disti <= rcutSq) in[0] = ti;
    }
    if (planeIntersect(d1, d2, halfl2, r_cm, P.s1, pcanglsw, ti, c, d)) {
        disti = (d <= 0) ? c * c : d * d + c * c;
        if (disti <= rcutSq) {
            if (in[0] == 0.0) in[0] = ti;
            else if (ti != in[0]) in[1] = ti;
        }
    }
    if (in[1] != 0.0) { io[0] = in[0]; io[1] = in[1]; return 2; }
    testIntrAtC(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, halfl2, in);
    if (in[1] == 0.0) {
        double3 v1 = mk(d1.x * halfl1 - r_cm.x, d1.y * halfl1 - r_cm.y, d1.z * halfl1 - r_cm.z);
        double3 v2 = mk(-d1.x * halfl1 - r_cm.x, -d1.y * halfl1 - r_cm.y, -d1.z * halfl1 - r_cm.z);
        capSphereIntersections(d1, d2, P, r_cm, in, pcanglsw, halfl1, halfl2, 2.0 * dot3(v1, d2), dot3(v1, v1) - rcutSq);
        capSphereIntersections(d1, d2, P, r_cm, in, pcanglsw, halfl1, halfl2, 2.0 * dot3(v2, d2), dot3(v2, v2) - rcutSq);
    } else {
        io[0] = in[0]; io[1] = in[1]; return 2;
    }
    if (in[1] == 0.0) {
        endInsideTest(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, halfl2, in);
        if (in[1] == 0.0) endInsideTest(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, -halfl2, in);
    }
    io[0] = in[0]; io[1] = in[1];
    return (in[1] == 0.0) ? 0 : 2;
}

// CPsc::cpscIntersect (paire.h:687-826): flat end caps instead of hemispheres.
static __device__ __noinline__ int cpscIntersect(double3 d1, double3 d2, PatchV P, double3 r_cm, double* io,
                                          double pcanglsw, double rcutSq, double halfl1, double halfl2) {
    double a, b, c, d, x1, disti, ti;
    double in[2] = {0, 0};
    double3 v1, v2;
    if (planeIntersect(d1, d2, halfl2, r_cm, P.s0, pcanglsw, ti, c, d)) {
        if (d <= 0) { disti = c * c; if (disti <= rcutSq) in[0] = ti; }
    }
    if (planeIntersect(d1, d2, halfl2, r_cm, P.s1, pcanglsw, ti, c, d)) {
        if (d <= 0) {
            disti = c * c;
            if (disti <= rcutSq) {
                if (in[0] == 0.0) in[0] = ti;
                else if (ti != in[0]) in[1] = ti;
            }
        }
    }
    if (in[1] != 0.0) { io[0] = in[0]; io[1] = in[1]; return 2; }
    testIntrAtC(d1, d2, P, r_cm, pcanglsw, rcutSq, halfl1, halfl2, in);
    if (in[1] == 0.0) {
        a = dot3(d1, d2);
        if (a != 0.0) {
#pragma unroll 1
            for (int cap = 0; cap < 2; ++cap) {
                double h = cap == 0 ? halfl1 : -halfl1;
                v1 = cap == 0 ? mk(r_cm.x + h * d1.x, r_cm.y + h * d1.y, r_cm.z + h * d1.z)
                              : mk(r_cm.x - halfl1 * d1.x, r_cm.y - halfl1 * d1.y, r_cm.z - halfl1 * d1.z);
                x1 = dot3(d1, v1) / a;
                if (!((x1 > halfl2) || (x1 < -halfl2))) {
                    v2 = mk(x1 * d2.x - v1.x, x1 * d2.y - v1.y, x1 * d2.z - v1.z);
                    b = dot3(v2, v2);
                    if (!(b > rcutSq)) testIntrPatch(d1, P.dir, v2, pcanglsw, x1, in);
                }
            }
        }
    } else {
        io[0] = in[0]; io[1] = in[1]; return 2;
    }
    if (in[1] == 0.0) {
#pragma unroll 1
        for (int end = 0; end < 2 && in[1] == 0.0; ++end) {
            v1 = end == 0 ? mk(d2.x * halfl2 - r_cm.x, d2.y * halfl2 - r_cm.y, d2.z * halfl2 - r_cm.z)
                          : mk(-d2.x * halfl2 - r_cm.x, -d2.y * halfl2 - r_cm.y, -d2.z * halfl2 - r_cm.z);
            a = dot3(v1, d1);
            v2 = mk(v1.x - d1.x * a, v1.y - d1.y * a, v1.z - d1.z * a);
            b = dot3(v2, v2);
            d = fabs(a) - halfl1;
            if (d <= 0) { if (b < rcutSq) testIntrPatch(d1, P.dir, v1, pcanglsw, end == 0 ? halfl2 : -1.0 * halfl2, in); }
        }
    }
    io[0] = in[0]; io[1] = in[1];
    return (in[1] == 0.0) ? 0 : 2;
}

// EPatch::atrE (scOOP/mc/paire.cpp:243-301): attraction of two intersecting patches, in two
// independent halves: the distance term of the intersection pieces (A: returns the
// cos^2 / plateau value, *f0 the length factor) and the angular switches and the parallel
// factor (B).  atrE = A * (((f0 * f1) * f2) * paral).
__device__ __forceinline__ double3 patchPieceVec(double3 d1, double3 d2, double3 r_cm, double S1, double S2, double T1,
                                                 double T2) {
    double3 a1 = scl((S1 + S2) * 0.5, d1), a2 = scl((T1 + T2) * 0.5, d2);
    return mk(a2.x - a1.x - r_cm.x, a2.y - a1.y - r_cm.y, a2.z - a1.z - r_cm.z);
}
static __device__ __noinline__ double patchAttractionA(const PairParam& ia, double3 d1, double3 d2, double3 r_cm,
                                                       double S1, double S2, double T1, double T2, double* f0out) {
    double v1 = fabs(S1 - S2), v2 = fabs(T1 - T2), f0 = 0.5 * (v1 + v2);
    double3 vi = patchPieceVec(d1, d2, r_cm, S1, S2, T1, T2);
    double3 md = minDistSegments(d1, d2, v1, v2, vi);
    double ndist = sqrt(dot3(md, md)), atr;
    if (ndist < ia.pdis) atr = -ia.epsilon;
    else { atr = cos(1.57079632679489661923132169163975 * (ndist - ia.pdis) / ia.pswitch); atr *= -atr * ia.epsilon; }
    *f0out = f0;
    return atr;
}
static __device__ __noinline__ void patchAttractionB(const PairParam& ia, double3 d1, double3 d2, double3 p1dir,
                                                     double3 p2dir, double3 r_cm, int pn1, int pn2, double S1,
                                                     double S2, double T1, double T2, double* f1out, double* f2out,
                                                     double* paralOut) {
    double3 vi = patchPieceVec(d1, d2, r_cm, S1, S2, T1, T2);
    double3 w = perpProj(vi, d1);
    double a = dot3(w, p1dir) / vlen(w);
    *f1out = fanglScale(a, ia.pcangl[0 + 2 * pn1], ia.pcanglsw[0 + 2 * pn1]);
    w = perpProj(neg3(vi), d2);
    a = dot3(w, p2dir) / vlen(w);
    *f2out = fanglScale(a, ia.pcangl[1 + 2 * pn2], ia.pcanglsw[1 + 2 * pn2]);
    double paral = 1.0;
    if (ia.parallel != 0.0) {   // EPatch::scparallel (paire.h:77-84)
        double cosa = dot3(d1, d2);
        if ((ia.parallel > 0 && cosa > 0) || (ia.parallel < 0 && cosa < 0)) paral = 1.0 + ia.parallel * cosa;
    }
    *paralOut = paral;
}
__device__ __forceinline__ double patchAttractionCombine(double atr, double f0, double f1, double f2, double paral) {
    atr *= f0 * f1 * f2 * paral;
    return atr;
}
static __device__ double patchAttraction(const PairParam& ia, double3 d1, double3 d2, double3 p1dir, double3 p2dir,
                                         double3 r_cm, int pn1, int pn2, double S1, double S2, double T1, double T2) {
    double f0, f1, f2, paral;
    double atr = patchAttractionA(ia, d1, d2, r_cm, S1, S2, T1, T2, &f0);
    patchAttractionB(ia, d1, d2, p1dir, p2dir, r_cm, pn1, pn2, S1, S2, T1, T2, &f1, &f2, &paral);
    return patchAttractionCombine(atr, f0, f1, f2, paral);
}

// x^-3 and x^-6 from one reciprocal: a few ulp from pow(x, -3) / pow(x, -6), with a
// dependent FP64 chain a third as long (FP64 latency dominates the move kernel).
__device__ __forceinline__ void invPow36(double x, double& i3, double& i6) {
    double r = 1.0 / x;
    i3 = r * r * r;
    i6 = i3 * i3;
}

// A r^-12 - B r^-6 from r (the Lennard-Jones part of WcaTrunc / Sca / WcaCos2Taylor).
__device__ __forceinline__ double lj12_6(double r, double A, double B) {
    double i6, i12;
    invPow36(r * r, i6, i12);
    return A * i12 - B * i6;
}

__device__ __forceinline__ double wcaTruncSq(double distSq, const PairParam& ia) {   // paire.h:385-393
    if (distSq > ia.rcutwcaSq) return 0.0;
    double i3, i6;
    invPow36(distSq, i3, i6);
    return ia.epsilon + ia.A * i6 - ia.B * i3;
}

// HarmonicSc (paire.h:239-280) between particle a and its bonded partner b.
static __device__ double bondSc(const PairParam& ia, const PView& a, const PView& b, double dist, const Con& con,
                         const double3& box) {
    const MolParam& m = *con.m;
    if (b.index == con.idx[1] || b.index == con.idx[0]) {
        bool tail = (b.index == con.idx[0]);
        double h1 = (ia.geotype[0] < SP) ? (ia.half_len[0] + (tail ? m.mod0 : m.mod1)) * (tail ? 1.0 : -1.0) : m.sp;
        double h2 = (ia.geotype[1] < SP) ? (ia.half_len[1] + (tail ? m.mod1 : m.mod0)) * (tail ? -1.0 : 1.0) : m.sp;
        double3 v1 = mk(a.pos.x + (a.dir.x * h1 / box.x), a.pos.y + (a.dir.y * h1 / box.y), a.pos.z + (a.dir.z * h1 / box.z));
        double3 v2 = mk(b.pos.x + (b.dir.x * h2 / box.x), b.pos.y + (b.dir.y * h2 / box.y), b.pos.z + (b.dir.z * h2 / box.z));
        v1 = imageVec(v1, v2, box);
        return harmonicE(sqrt(dot3(v1, v1)), m.eq0, m.c0);
    }
    if (b.index == con.idx[2] || b.index == con.idx[3]) return harmonicE(dist, m.eq1, m.c1);
    return 0.0;
}

static __device__ double angle2Of(const PView& p, const PView& q) {   // AngleSc::angleEnergyAngle2 (paire.h:340-352)
    double3 ax = cross3(p.dir, q.dir);
    double3 x1 = cross3(p.dir, ax), x2 = cross3(q.dir, ax);
    double3 ppd = ld3(p.patch->pd[0]), qpd = ld3(q.patch->pd[0]);
    double v1x = dot3(x1, ppd), v1y = dot3(ax, ppd), v2x = dot3(x2, qpd), v2y = dot3(ax, qpd);
    return acos((v1x * v2x + v1y * v2y) / (sqrt((v1x * v1x + v1y * v1y) * (v2x * v2x + v2y * v2y))));
}

// AngleSc (paire.h:283-337).
static __device__ double angleSc(const PairParam& ia, const PView& a, const PView& b, const Con& con, const double3& box) {
    const MolParam& m = *con.m;
    bool partner = (b.index == con.idx[0] || b.index == con.idx[1]);
    if (!partner) return 0.0;
    bool tail = (b.index == con.idx[0]);
    double e = 0.0;
    if (m.angle1c >= 0) {
        double3 v1, v2;
        if (ia.geotype[0] < SP) v1 = a.dir;
        else {
            double h = ia.half_len[1] * (tail ? -1.0 : 1.0);
            v1 = mk(b.pos.x + b.dir.x * h / box.x, b.pos.y + b.dir.y * h / box.y, b.pos.z + b.dir.z * h / box.z);
            v1 = imageVec(v1, a.pos, box);
            normalise3(v1);
        }
        if (ia.geotype[1] < SP) v2 = b.dir;
        else {
            double h = ia.half_len[0] * (tail ? 1.0 : -1.0);
            v2 = mk(a.pos.x + a.dir.x * h / box.x, a.pos.y + a.dir.y * h / box.y, a.pos.z + a.dir.z * h / box.z);
            v2 = imageVec(v2, b.pos, box);
            normalise3(v2);
        }
        e += harmonicE(acos(dot3(v1, v2)), m.angle1eq, m.angle1c);
    }
    if (m.angle2c >= 0 && ia.geotype[0] < SP && ia.geotype[1] < SP) {
        double ang = tail ? angle2Of(b, a) : angle2Of(a, b);
        e += harmonicE(ang, m.angle2eq, m.angle2c);
    }
    return e;
}

__device__ __forceinline__ double bondedTerms(const PairParam& ia, const PView& a, const PView& b, double dist,
                                              const Con& con, const double3& box) {
    if (con.isEmpty) return 0.0;
    bool isPartner = (b.index == con.idx[0] || b.index == con.idx[1] || b.index == con.idx[2] || b.index == con.idx[3]);
    if (!isPartner) return 0.0;
    double e = bondSc(ia, a, b, dist, con, box);
    e += angleSc(ia, a, b, con, box);
    return e;
}

// The three independent FP64 chains of a single-patch PSC/CPSC pair (scScEnergy below
// with one patch combination), for evaluation by three threads side by side:
//   role 0: closest segment distance and the WCA term, returns 0.0 + rep (no bond terms:
//           callers pass non-bonded pairs only), *ok = the attractive branch is on;
//   role 1: intersections of particle 2's axis with particle 1's patch (T, return na);
//   role 2: intersections of particle 1's axis with particle 2's patch (S, return nb).
// The pair energy is then  e0 + patchAttraction(...)  when ok && na >= 2 && nb >= 2, else
// e0 + 0.0: bit-identical to scScEnergy, which evaluates the same chains in sequence.
__device__ __forceinline__ double simpleScRole0(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                                int* ok) {
    double3 md = minDistSegments(a.dir, b.dir, ia.half_len[0], ia.half_len[1], r_cm);
    double distSq = dot3(md, md);
    double rep = wcaTruncSq(distSq, ia);
    *ok = !((distSq > ia.rcutSq) || (ia.epsilon == 0.0) || ia.exclude);
    return 0.0 + rep;
}
__device__ __forceinline__ int simpleScRole1(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                             double* T) {
    PatchV P1{ld3(a.patch->pd[0]), ld3(a.patch->ps[0]), ld3(a.patch->ps[1])};
    return ia.firstPsc ? pscIntersect(a.dir, b.dir, P1, r_cm, T, ia.pcanglsw[0], ia.rcutSq, ia.half_len[0], ia.half_len[1])
                       : cpscIntersect(a.dir, b.dir, P1, r_cm, T, ia.pcanglsw[0], ia.rcutSq, ia.half_len[0], ia.half_len[1]);
}
__device__ __forceinline__ int simpleScRole2(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                             double* S) {
    PatchV P2{ld3(b.patch->pd[0]), ld3(b.patch->ps[0]), ld3(b.patch->ps[1])};
    double3 mr = neg3(r_cm);
    return ia.secondPsc ? pscIntersect(b.dir, a.dir, P2, mr, S, ia.pcanglsw[1], ia.rcutSq, ia.half_len[1], ia.half_len[0])
                        : cpscIntersect(b.dir, a.dir, P2, mr, S, ia.pcanglsw[1], ia.rcutSq, ia.half_len[1], ia.half_len[0]);
}
__device__ __forceinline__ double simpleScCombine(const PairParam& ia, const PView& a, const PView& b,
                                                  const double3& r_cm, double e0, int ok, int na, int nb, const double* T,
                                                  const double* S) {
    double atr = 0.0;
    if (ok && na >= 2 && nb >= 2)
        atr += patchAttraction(ia, a.dir, b.dir, ld3(a.patch->pd[0]), ld3(b.patch->pd[0]), r_cm, 0, 0, S[0], S[1], T[0],
                               T[1]);
    return e0 + atr;
}
// The attraction's two halves of a single-patch pair (for two threads), and the sum.
__device__ __forceinline__ double simpleScAttrA(const PairParam& ia, const PView& a, const PView& b,
                                                const double3& r_cm, const double* T, const double* S, double* f0) {
    return patchAttractionA(ia, a.dir, b.dir, r_cm, S[0], S[1], T[0], T[1], f0);
}
__device__ __forceinline__ void simpleScAttrB(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                              const double* T, const double* S, double* f1, double* f2,
                                              double* paral) {
    patchAttractionB(ia, a.dir, b.dir, ld3(a.patch->pd[0]), ld3(b.patch->pd[0]), r_cm, 0, 0, S[0], S[1], T[0], T[1],
                     f1, f2, paral);
}
__device__ __forceinline__ double simpleScSum(double e0, bool attractive, double atrA, double f0, double f1, double f2,
                                              double paral) {
    double atr = 0.0;
    if (attractive) atr += patchAttractionCombine(atrA, f0, f1, f2, paral);
    return e0 + atr;
}

// Patch combination c (pn1 = c & 1, pn2 = c >> 1) of an SC-SC pair of patchy types: its two
// intersection chains and the halves of its attraction, for evaluation by separate threads
// (the scScEnergy loop below evaluates the same chains in sequence; a combination counts
// when the attractive branch is on and both intersections give 2 points).
__device__ __forceinline__ bool comboValid(const PairParam& ia, int c) {
    int pn1 = c & 1, pn2 = c >> 1;
    return !((pn1 && !ia.fT) || (pn2 && !ia.sT));
}
__device__ __forceinline__ void comboAxes(const PairParam& ia, const PView& a, const PView& b, int c, double3& d1,
                                          double3& d2) {
    int pn1 = c & 1, pn2 = c >> 1;
    d1 = ia.fCH ? ld3(a.patch->ch[pn1]) : a.dir;
    d2 = ia.sCH ? ld3(b.patch->ch[pn2]) : b.dir;
}
__device__ __forceinline__ int comboIntersect1(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                               int c, double* T) {
    int pn1 = c & 1;
    double3 d1, d2;
    comboAxes(ia, a, b, c, d1, d2);
    PatchV P1{ld3(a.patch->pd[pn1]), ld3(a.patch->ps[2 * pn1]), ld3(a.patch->ps[2 * pn1 + 1])};
    return ia.firstPsc
        ? pscIntersect(d1, d2, P1, r_cm, T, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1])
        : cpscIntersect(d1, d2, P1, r_cm, T, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1]);
}
__device__ __forceinline__ int comboIntersect2(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                               int c, double* S) {
    int pn2 = c >> 1;
    double3 d1, d2;
    comboAxes(ia, a, b, c, d1, d2);
    PatchV P2{ld3(b.patch->pd[pn2]), ld3(b.patch->ps[2 * pn2]), ld3(b.patch->ps[2 * pn2 + 1])};
    double3 mr = neg3(r_cm);
    return ia.secondPsc
        ? pscIntersect(d2, d1, P2, mr, S, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0])
        : cpscIntersect(d2, d1, P2, mr, S, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0]);
}
__device__ __forceinline__ double comboAttrA(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                             int c, const double* T, const double* S, double* f0) {
    double3 d1, d2;
    comboAxes(ia, a, b, c, d1, d2);
    return patchAttractionA(ia, d1, d2, r_cm, S[0], S[1], T[0], T[1], f0);
}
__device__ __forceinline__ void comboAttrB(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                           int c, const double* T, const double* S, double* f1, double* f2,
                                           double* paral) {
    int pn1 = c & 1, pn2 = c >> 1;
    double3 d1, d2;
    comboAxes(ia, a, b, c, d1, d2);
    patchAttractionB(ia, d1, d2, ld3(a.patch->pd[pn1]), ld3(b.patch->pd[pn2]), r_cm, pn1, pn2, S[0], S[1], T[0], T[1],
                     f1, f2, paral);
}
// The WCA chain of a patchy SC-SC pair: returns 0.0 + rep (callers pass non-bonded pairs),
// *ok = the attractive branch is on.
__device__ __forceinline__ double patchyWca(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                            int* ok) {
    return simpleScRole0(ia, a, b, r_cm, ok);
}

// SC-SC pair (SpheroCylinder::operator(), paire.h:1122-1196).
static __device__ __noinline__ double scScEnergy(const PairParam& ia, const PView& a, const PView& b, const double3& r_cm,
                                          double dist, const Con& con, const double3& box, unsigned* bits,
                                          double* dsqOut) {
    double abE = bondedTerms(ia, a, b, dist, con, box);
    double3 md = minDistSegments(a.dir, b.dir, ia.half_len[0], ia.half_len[1], r_cm);
    double distSq = dot3(md, md);
    *dsqOut = distSq;
    double rep = wcaTruncSq(distSq, ia);
    if (!(distSq > ia.rcutwcaSq)) *bits |= V_WCA;
    double atr = 0.0;
    if (!((distSq > ia.rcutSq) || (ia.epsilon == 0.0) || ia.exclude)) {
        *bits |= V_ATR;
        if (ia.kind != K_SC_SCN) {
#pragma unroll 1
            for (int c = 0; c < 4; ++c) {
                int pn1 = c & 1, pn2 = c >> 1;
                if ((pn1 && !ia.fT) || (pn2 && !ia.sT)) continue;
                double3 d1 = ia.fCH ? ld3(a.patch->ch[pn1]) : a.dir;
                double3 d2 = ia.sCH ? ld3(b.patch->ch[pn2]) : b.dir;
                if (ia.kind == K_SC_SCA) {      // Sca::operator() (paire.h:845-852)
                    double3 m2 = minDistSegments(d1, d2, ia.half_len[0], ia.half_len[1], r_cm);
                    double dd = sqrt(dot3(m2, m2));
                    if (!(dd > ia.rcutwca)) atr += lj12_6(dd, ia.A, ia.B) + ia.epsilon;
                    continue;
                }
                PatchV P1{ld3(a.patch->pd[pn1]), ld3(a.patch->ps[2 * pn1]), ld3(a.patch->ps[2 * pn1 + 1])};
                double T[2] = {0, 0}, S[2] = {0, 0};
                int na = ia.firstPsc
                    ? pscIntersect(d1, d2, P1, r_cm, T, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1])
                    : cpscIntersect(d1, d2, P1, r_cm, T, ia.pcanglsw[2 * pn1], ia.rcutSq, ia.half_len[0], ia.half_len[1]);
                if (na < 2) continue;
                *bits |= 1u << (8 + 2 * c);
                PatchV P2{ld3(b.patch->pd[pn2]), ld3(b.patch->ps[2 * pn2]), ld3(b.patch->ps[2 * pn2 + 1])};
                double3 mr = neg3(r_cm);
                int nb = ia.secondPsc
                    ? pscIntersect(d2, d1, P2, mr, S, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0])
                    : cpscIntersect(d2, d1, P2, mr, S, ia.pcanglsw[2 * pn2 + 1], ia.rcutSq, ia.half_len[1], ia.half_len[0]);
                if (nb < 2) continue;
                *bits |= 1u << (9 + 2 * c);
                atr += patchAttraction(ia, d1, d2, P1.dir, P2.dir, r_cm, pn1, pn2, S[0], S[1], T[0], T[1]);
            }
        }
    }
    return abE + rep + atr;
}

// MixSpSc::closestDist (paire.h:1077-1093): point to segment.
__device__ __forceinline__ double pointSegment(const double3& rc, const double3& d1, double halfl, double& contt, double3& dv) {
    contt = dot3(d1, rc);
    double d = -halfl;
    if (contt >= halfl) d = halfl;
    else if (contt > -halfl) d = contt;
    dv = mk(-rc.x + d1.x * d, -rc.y + d1.y * d, -rc.z + d1.z * d);
    return dot3(dv, dv);
}

// PscSpa / CPscSpa / ScaSpa (paire.h:911-1010).
static __device__ double patchToSphere(int kind, double dist, double contt, const double3& distvec, const PairParam& ia,
                                const double3& d1, const double3& pdir) {
    double atr;
    if (dist < ia.pdis) atr = -ia.epsilon;
    else { atr = cos(1.57079632679489661923132169163975 * (dist - ia.pdis) / ia.pswitch); atr *= -atr * ia.epsilon; }
    double a = 0.0;
    if (kind != K_MIX_SCA_SPA) {
        double3 w = perpProj(distvec, d1);
        a = dot3(w, pdir) / vlen(w);
    }
    double halfl = ia.half_len[0];
    double b = sqrt(ia.rcutSq - dist * dist), f0;
    if (contt + b > halfl) f0 = halfl; else f0 = contt + b;
    if (contt - b < -halfl) f0 -= -halfl; else f0 -= contt - b;
    if (kind == K_MIX_SCA_SPA) atr *= f0;
    else atr *= fanglScale(a, ia.pcangl[0], ia.pcanglsw[0]) * (f0);
    return atr;
}

// SC-sphere pair (MixSpSc::operator(), paire.h:1022-1067).  iap is the entry with the SC first.
static __device__ __noinline__ double scSphereEnergy(const PairParam& ia, const PairParam& iap, const PView& a, const PView& b,
                                              const double3& r_cm, double dist, const Con& con, const double3& box,
                                              unsigned* bits, double* dsqOut) {
    bool isp1Spc = (ia.geotype[0] < SP);
    const PView& spc = isp1Spc ? a : b;
    double3 rc = isp1Spc ? r_cm : neg3(r_cm);
    double contt = 0.0;
    double3 dv;
    double distSq = pointSegment(rc, spc.dir, iap.half_len[0], contt, dv);
    *dsqOut = distSq;
    double abE = bondedTerms(ia, a, b, dist, con, box);
    double rep = 0.0, atr = 0.0;
    if (distSq < iap.rcutwcaSq) { rep = wcaTruncSq(distSq, ia); *bits |= V_WCA; }
    bool isFar = (ia.kind == K_MIX_CPSC_SP) && ((contt > iap.half_len[0]) || (contt < -iap.half_len[0]));
    if (isFar) *bits |= V_FAR;
    if (!((distSq > iap.rcutSq) || (iap.epsilon == 0.0) || iap.exclude || isFar)) {
        *bits |= V_ATR;
        bool chiral = iap.mixChiral, sec = iap.mixSec;
        double3 axis0 = chiral ? ld3(spc.patch->ch[0]) : spc.dir;
        if (chiral) distSq = pointSegment(rc, axis0, iap.half_len[0], contt, dv);
        double dd = sqrt(distSq);
        if (dd < iap.rcut) {
            *bits |= 1u << 8;
            atr = patchToSphere(ia.kind, dd, contt, dv, iap, axis0, ld3(spc.patch->pd[0]));
        }
        if (sec) {
            double3 axis1 = chiral ? ld3(spc.patch->ch[1]) : spc.dir;
            distSq = pointSegment(rc, axis1, iap.half_len[0], contt, dv);
            dd = sqrt(distSq);
            if (dd < iap.rcut) {
                *bits |= 1u << 9;
                atr += patchToSphere(ia.kind, dd, contt, dv, iap, axis1, ld3(spc.patch->pd[1]));
            }
        }
    }
    return abE + rep + atr;
}

// Sphere pairs (Sphere<WcaTrunc / WcaCos2Taylor, HarmonicSp>, paire.h:1099-1109, 376-439).
static __device__ __noinline__ double sphereEnergy(const PairParam& ia, const PView& b, double dist, const Con& con,
                                            unsigned* bits) {
    double bond = 0.0;
    if (!con.isEmpty) {     // HarmonicSp (paire.h:221-236)
        if (b.index == con.idx[1] || b.index == con.idx[0]) bond = harmonicE(dist, con.m->eq0, con.m->c0);
        else if (b.index == con.idx[2] || b.index == con.idx[3]) bond = harmonicE(dist, con.m->eq1, con.m->c1);
    }
    double pot = 0.0;
    if (ia.kind == K_SP_WCA) {
        if (!(dist > ia.rcutwca)) { pot = lj12_6(dist, ia.A, ia.B) + ia.epsilon; *bits |= V_WCA; }
    } else if (!(dist > ia.rcut || ia.epsilon == 0.0 || ia.exclude)) {
        *bits |= V_ATR;
        double e;
        if (dist > ia.pdis) {
            // degree-16 Taylor cos^2 of WcaCos2Taylor, term order kept
            e = 1.57079632679489661923132169163975 * (dist - ia.pdis) * ia.pswitchINV;
            e *= e;
            e = (1 - e + e * e * (1.0 / 3.0) - e * e * e * (2.0 / 45.0) + e * e * e * e * (1.0 / 315.0) -
                 e * e * e * e * e * (2.0 / 14175.0) + e * e * e * e * e * e * (2.0 / 467775.0) -
                 e * e * e * e * e * e * e * (4.0 / 42567525) + e * e * e * e * e * e * e * e * (1.0 / 638512875)) *
                -ia.epsilon;
        } else {
            e = -ia.epsilon;
        }
        if (dist > ia.rcutwca) pot = e;
        else { pot = lj12_6(dist, ia.A, ia.B); *bits |= V_WCA; }
    }
    return bond + pot;
}

// Energy of the evaluated pair (a, b) given r_cm = image(a, b) and r^2; the caller
// has applied the PairE prefilter (r^2 > sqmaxcut with an empty conlist -> 0).
__device__ __forceinline__ double pairBody(const DevCtx& c, const PView& a, const PView& b, const double3& r_cm,
                                           double dotrcm, const Con& con, const double3& box, unsigned* bits,
                                           double* dsq) {
    *bits |= V_EVAL;
    double dist = sqrt(dotrcm);
    const PairParam& ia = c.params[a.type * c.ntypes + b.type];
    int kind = ia.kind;
    if (kind >= K_SC_PSC_CPSC && kind <= K_SC_SCA) return scScEnergy(ia, a, b, r_cm, dist, con, box, bits, dsq);
    if (kind >= K_MIX_SCA_SPA) {
        const PairParam& iap = (ia.geotype[0] < SP) ? ia : c.params[b.type * c.ntypes + a.type];
        return scSphereEnergy(ia, iap, a, b, r_cm, dist, con, box, bits, dsq);
    }
    if (kind == K_SP_WCA || kind == K_SP_SPA) { *dsq = dotrcm; return sphereEnergy(ia, b, dist, con, bits); }
    return 0.0;   // EBasic (paire.h:207-213)
}

// PairE::operator() (paire.h:1209-1220) for particle a against b.
__device__ __forceinline__ double pairEnergy(const DevCtx& c, const PView& a, const PView& b, const Con& con,
                                             const double3& box, unsigned* bits, double* dsq) {
    *bits = 0;
    *dsq = -1.0;
    double3 r_cm = imageVec(a.pos, b.pos, box);
    double dotrcm = dot3(r_cm, r_cm);
    if (dotrcm > c.sqmaxcut && con.isEmpty) return 0.0;
    return pairBody(c, a, b, r_cm, dotrcm, con, box, bits, dsq);
}

// ConList of particle i from its molecule record (Conf.h:97-146).
__device__ __forceinline__ Con makeCon(const DevCtx& c, int i, int4 mol) {
    Con con;
    con.idx[0] = con.idx[1] = con.idx[2] = con.idx[3] = -1;
    con.isEmpty = 1;
    con.m = &c.mols[mol.x];
    int size = mol.z, pos = mol.y;
    if (size > 1) {
        if (con.m->bonded) {
            if (pos > 0) con.idx[0] = i - 1;
            if (pos + 1 < size) con.idx[1] = i + 1;
            con.isEmpty = 0;
        }
        if (con.m->bonded2) {
            if (pos > 1) con.idx[2] = i - 2;
            if (pos + 2 < size) con.idx[3] = i + 2;
            con.isEmpty = 0;
        }
    }
    return con;
}

__device__ __forceinline__ Con emptyCon(const DevCtx& c) {
    Con con;
    con.idx[0] = con.idx[1] = con.idx[2] = con.idx[3] = -1;
    con.isEmpty = 1;
    con.m = c.mols;
    return con;
}

}  // namespace scg
