/* sc_oracle.h -- CPU oracle for the SC Metropolis hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of the reference's
 * pair energy, one-particle / total energy and single-particle move loop (with its volume,
 * type switch and grand-canonical moves)
 * (robertvacha/SC, scOOP/mc/paire.h, paire.cpp, totalenergycalculator.h,
 * movecreator.cpp, updater.cpp, structures/topo.cpp, particle.*), used by the
 * tests as the reference to compare against and by bench.py as the timed CPU baseline.  The product
 * (sc_gb300/) never includes, links or loads it.
 *
 * Parity is pinned: tests/test_oracle_golden.py compares every function below
 * with golden vectors produced by the reference itself (oracle/ref_dump.cpp,
 * built from the reference's own sources by oracle/Makefile).
 */
#ifndef SC_ORACLE_H
#define SC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAXT 40

typedef struct { double x, y, z; } or_vec;

/* One entry of the reference's Ia_param table (scOOP/structures/structures.h:187-254). */
typedef struct {
    int geotype[2];
    int exclude;
    int pad_;
    double sigma, epsilon, A, B, pdis, pswitch, pswitchINV;
    double pcangl[4], pcanglsw[4];
    double rcut, rcutSq, rcutwca, rcutwcaSq;
    double pcoshalfi[4], psinhalfi[4];
    double csecpatchrot[2], ssecpatchrot[2];
    double volume;
    double len[2], half_len[2];
    double chiral_cos[2], chiral_sin[2];
    double parallel;
} or_param;

/* Raw per-type line of the [Types] section of top.init (scOOP/mc/inicializer.cpp:660-852). */
typedef struct {
    int type;          /* type number 0..39 */
    int geotype;       /* SC codes: SCN=10 .. TCHCPSC=19, SPN=30, SPA=31 */
    int nfields;       /* numeric fields after EPSILON SIGMA (inicializer.cpp:688) */
    int pad_;
    double param[12];  /* eps, sigma, pdis, pswitch, pangl, panglsw, len, parallel, secrot|chiral, pangl2, panglsw2, chiral */
} or_type_in;

/* Particle (scOOP/structures/particle.h:24-37), positions in box fractions. */
typedef struct {
    or_vec pos, dir, pd[2], ps[4], ch[2];
    int type, molType;
} or_particle;

/* Molecule type (scOOP/structures/moleculeparams.h:10-79) with its place in the particle vector. */
typedef struct {
    int size, first, count, pad_;
    double bond1c, bond1eq, bond2c, bond2eq, bonddc, bonddeq, bondhc, bondheq;
    double angle1c, angle1eq, angle2c, angle2eq;
} or_moltype;

typedef struct {
    int n;
    int nmol;
    or_particle* p;
    const or_moltype* mols;
    const or_param* params;   /* OR_MAXT*OR_MAXT, row-major [t1][t2] */
    double box[3];
    double sqmaxcut;
} or_system;

/* Verdict bits, shared with the CUDA kernels' layout. */
enum {
    OR_V_EVAL = 1u << 0, OR_V_WCA = 1u << 1, OR_V_ATR = 1u << 2, OR_V_FAR = 1u << 3
};

double or_pair_energy(const or_system* s, int i, int j, unsigned* bits, double* distSq);
double or_one_to_all(const or_system* s, int target);
double or_all_to_all(const or_system* s);
double or_mol2others(const or_system* s, int first, int size);
/* Nematic order S2 (largest eigenvalue of <3/2 u u^T - 1/2 I> over the spherocylinders'
 * axes) and the director (may be NULL); no counterpart in the reference. */
int or_nematic(const or_system* s, double* s2, double dir[3]);
/* PairE over a batch of ordered pairs (bits, dsq may be NULL). */
void or_pair_energies(const or_system* s, long n, const int* I, const int* J, double* E, unsigned* bits, double* dsq);
/* The ordered pairs (i a target, or any particle when targets is NULL; j != i) that PairE's
 * prefilter admits (paire.h:1209-1215): image distance^2 <= sqmaxcut, or j bonded to i.
 * At most cap written; *count = all of them. */
void or_prefilter_pairs(const or_system* s, int nt, const int* targets, long cap, int* I, int* J, long* count);

int or_derive_params(const or_type_in* types, int ntypes, const unsigned char* exclusions /* 40x40 or NULL */,
                     or_param* out /* 40x40 */, double* sqmaxcut, double* maxcut);
void or_particle_init(or_particle* p, const or_param* diag);
void or_psc_rotate(or_particle* p, int geotype, double angle, or_vec axis, int positive);

typedef struct {
    long nsweeps;
    long seed;
    double temper, press, shave, chainprob;
    double transmx;      /* full displacement length, already doubled as sim.h:365 does */
    double rot_angle;    /* half-angle bound, rotmx/180*PI/4 as sim.h:359 */
    double edge_mx;      /* full edge change range, already doubled */
    double chainmmx, chainr_angle;
    int ptype;
    int pairlist_update; /* 0: brute force; k: Verlet list rebuilt every k sweeps */
    long max_moves;      /* stop after this many attempted moves (0: no bound) */
    int energy_matrix;   /* 1: TotalEMatrix (old energies from the stored pair energies, the reference's
                            default); 0: TotalEFull (old and new energies by pair evaluation) */
    int pad_;
    /* chain moves (MoveCreator::chainMove, movecreator.cpp:305-328) are chosen with probability
     * chainprob per step after the volume move's shprob (updater.cpp:215-218), displacing a
     * random chain by chainmmx or turning it by up to chainr_angle (a quaternion half-angle);
     * type switching (MoveCreator::switchTypeMove, movecreator.cpp:233-303) with probability
     * switchprob after those (updater.cpp:219-222); the arrays are per particle, NULL without
     * switching */
    double switchprob;
    int* switch_other;       /* the other type of the particle's switch pair, -1 for none (swapped by moves) */
    const int* switch_dmu;   /* delta_mu as the reference's move reads it (an int) */
    int* switched;           /* 1 while the particle is in its switch type (updated by moves) */
    /* grand-canonical moves (MoveCreator::muVTMove, movecreator.cpp:797-924), one after every
     * grand_every-th sweep (updater.cpp:164-179), for n_gc single-particle species; the system's
     * particle array holds gc_cap slots and its n, and the molecule records' first / count,
     * follow the moves (not combined with switching) */
    int grand_every, n_gc, gc_cap, pad2_;
    const int* gc_moltype;   /* molecule type of each species */
    const int* gc_type;      /* its particle type */
    const double* gc_chempot;   /* log(activity Nav 1e-24) (inicializer.cpp:1094) */
} or_mc_opts;

typedef struct {
    long moves, acc_trans, rej_trans, acc_rot, rej_rot, acc_vol, rej_vol, acc_chain, rej_chain;
    double energy;       /* running total energy */
    double energy_start;
    double seconds;
    long acc_switch, rej_switch;
    long acc_insert, rej_insert, acc_delete, rej_delete;
} or_mc_stats;

int or_mc_run(or_system* s, const or_mc_opts* o, or_mc_stats* st);

/* The same loop as a resumable state, so that the moves can be timed apart from the set-up
 * the reference does before its timed loop (initial energy / energy matrix, first pair
 * list).  Volume moves follow every coupling of pressureMove (ptype 0..5), undone on
 * rejection by the reference's own subtraction.  or_mc_open returns NULL for an empty system
 * without grand-canonical species, a ptype outside 0..5, or grand-canonical moves together
 * with switching;
 * or_mc_advance runs `moves` more steps and adds to *st (moves, acceptances, seconds). */
typedef struct or_mc or_mc;
or_mc* or_mc_open(or_system* s, const or_mc_opts* o);
int or_mc_advance(or_mc* m, long moves, or_mc_stats* st);
/* Runs the rest of the current sweep and then sweeps-1 more (grand-canonical runs count sweeps,
 * since their particle count changes between sweeps). */
int or_mc_sweeps(or_mc* m, long sweeps, or_mc_stats* st);
double or_mc_energy(const or_mc* m);
double or_mc_setup_seconds(const or_mc* m);
void or_mc_close(or_mc* m);

/* Wang-Landau table and walker state of or_wl_run. */
typedef struct {
    int wlm[2];
    int len[2];            /* bins per order parameter (len[1] = 1 for one) */
    double minorder[2], dorder[2];
    double alpha;
    double* weights;       /* len[0] * len[1], order 0 fastest; updated in place */
    long* hist;
    long cur[2];           /* current bins (set by the caller, e.g. from or_wl_orders) */
    long updates;
    int converged;
    int wlmtype;           /* the particle type of orders 2 and 7 (options wlmtype) */
} or_wl;

/* The reference's sequential loop with a Wang-Landau bias (single-particle moves; volume
 * moves of every coupling, ptype 0..5, with probability shave / N per step; order parameters
 * 1, 2, 3, 4, 7, 8, 9), WangLandau::run / runRot / runPress / accept / reject / update.
 * Returns -2 for a ptype outside 0..5, -3 for orders 5 / 6 or a mesh without squares, -1 for
 * an empty system, else 0. */
int or_wl_run(or_system* s, const or_mc_opts* o, or_wl* wl, or_mc_stats* st);

/* Wang-Landau starting bins (WangLandau::init, scOOP/mc/wanglandau.cpp:49-137) of order
 * parameters 1, 2, 3, 4, 7, 8, 9 (wlmtype: the particle type of the mesh and contact orders),
 * with the system centre and sysvolume they use. */
int or_wl_orders(const or_system* s, const int wlm[2], int wlmtype, const double minorder[2], const double dorder[2],
                 long out[2], double syscm[3], double* sysvolume);

#ifdef __cplusplus
}
#endif
#endif
