/* sc_gb300.h -- C ABI of the GB300 Metropolis hot path for patchy spherocylinders.
 *
 * Drop-in boundary for the energy / move path of SC (robertvacha/SC, "scOOP").
 * The reference binds this path at compile time, not through an FFI:
 *     typedef TotalEMatrix<PairE> TotalEnergyCalculator;   scOOP/mc/totalenergycalculator.h:1227
 * consumed by Updater (scOOP/mc/updater.h:33) and MoveCreator (scOOP/mc/movecreator.h:15,36)
 * through the TotalE virtual interface (totalenergycalculator.h:136-297).  Each
 * entry point below names the reference call it replaces.
 *
 * Conventions
 *   - Every call returns SC_OK (0) or a negative SC_ERR_* code; sc_last_error()
 *     returns a message for the calling thread.  Nothing here exits the process.
 *   - Plain pointers and sizes only; host buffers belong to the caller.
 *   - One context = one system on one CUDA device and one stream.  A context is
 *     not shared between threads.  Every call makes the context's device current
 *     while it runs and restores the calling thread's current device on return.
 *   - Positions are box fractions (the reference's internal coordinates),
 *     energies in the reference's units (kT/epsilon scale of top.init).
 */
#ifndef SC_GB300_H
#define SC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SC_OK 0
#define SC_ERR_ARG (-1)        /* bad argument (null pointer, index out of range) */
#define SC_ERR_IO (-2)         /* a file could not be read or written */
#define SC_ERR_PARSE (-3)      /* options / top.init / config.init rejected */
#define SC_ERR_CUDA (-4)       /* a CUDA call failed (no device, launch error) */
#define SC_ERR_RANGE (-5)      /* a size beyond a documented maximum */
#define SC_ERR_STATE (-6)      /* call not valid in the current state */
#define SC_ERR_UNSUPPORTED (-7) /* input outside the GPU path (see sc_last_error) */
#define SC_ERR_DEVICE (-8)     /* a kernel reported an error status (e.g. a dataflow wait that gave up) */

typedef struct sc_context sc_context;

/* Derived interaction parameters of one type pair: the fields of the reference's
 * Ia_param (scOOP/structures/structures.h:187-254) that the energy uses. */
typedef struct {
    int geotype[2];
    int exclude;
    int kind;            /* pair functor chosen as in PairE::initIntFCE (scOOP/mc/paire.cpp:6-80) */
    double sigma, epsilon, A, B, pdis, pswitch, pswitchINV;
    double pcangl[4], pcanglsw[4];
    double rcut, rcutSq, rcutwca, rcutwcaSq;
    double pcoshalfi[4], psinhalfi[4];
    double csecpatchrot[2], ssecpatchrot[2];
    double volume;
    double len[2], half_len[2];
    double chiral_cos[2], chiral_sin[2];
    double parallel;
} sc_pair_param;

/* State of one particle, as Particle (scOOP/structures/particle.h:24-37). */
typedef struct {
    double pos[3];        /* box fractions */
    double dir[3];
    double patchdir[2][3];
    double patchsides[4][3];
    double chdir[2][3];
    int type;
    int molType;
} sc_particle;

/* Move-loop parameters: the options-file values of Sim (scOOP/structures/sim.h:15-70) the
 * loop uses, after the unit conversions of sim.h:359-381.  sc_default_run() fills them
 * from the options file of the context. */
typedef struct {
    long nsweeps;
    unsigned long long seed;
    double temper;
    double press;
    int ptype;              /* pressure coupling of volume moves (movecreator.cpp:330-546): 0 one random
                               edge, 1 isotropic, 2 xy with z fixed, 3 xy at fixed volume, 4 x (the
                               reference's xy branch), 5 y only */
    int volume_every;       /* sweeps between volume moves (options shave=1 -> every sweep); 0: none (NVT) */
    double transmx;         /* displacement length (already doubled, sim.h:365) */
    double rot_angle;       /* half-angle bound of pscRotate (rotmx/180*PIH*0.5, sim.h:359) */
    double edge_mx;         /* full edge-change range (already doubled, sim.h:363) */
    double chainprob;       /* chain moves per particle move (0: none) */
    double chainmmx;        /* chain displacement length (already doubled) */
    double chain_angle;     /* chain rotation angle bound, radians */
    int check_every;        /* sweeps between exact total-energy checks (0: none) */
    int time_phases;        /* 1: time the move kernels with CUDA events (adds events to the stream) */
    int stencil;            /* cell-list reach s: cells >= maxcut/s wide, (s+1)^3 colours; 0: chosen by the tuner */
    int delayed;            /* 1: two-stage moves with the context's surrogate (sc_set_surrogate) as first stage */
    int variant;            /* move kernel, bit 0: more moves in flight per SM (large systems), else lowest
                               latency per move; bit 1: paired passes (two moves per stage C); bit 2: one
                               dataflow launch per sweep instead of one launch per colour; bit 3: the
                               dataflow sweep with one warp per cell (plain moves, no Wang-Landau
                               weights; bits 1 and 2 then ignored); -1: the reach
                               and variant sc_tune measured fastest for this context (stencil 0 takes
                               the tuned reach), else the dataflow sweep */
    int flow_wait_polls;    /* dataflow sweep: polls of one wait for a neighbouring cell before the
                               kernel gives up and the call returns SC_ERR_DEVICE (0: 2^19, about
                               0.2 s; a wait in a sound run lasts well under 20 ms) */
    int grand_every;        /* sweeps between grand-canonical insert / delete moves (options
                               nGrandCanon; MoveCreator::muVTMove, movecreator.cpp:797-924); 0: none.
                               Needs top.init ACTIVITY species; replicas add the grand-canonical
                               term to their exchanges (movecreator.cpp:728-734) */
    long sweep_offset;      /* sweeps the caller's loop ran before this call: a move due every
                               grand_every sweeps follows sweep k of the loop when k % grand_every
                               == 0 (updater.cpp:165), k counted from the loop's start */
    double switchprob;      /* type switch attempts per particle move (options switchprob;
                               MoveCreator::switchTypeMove, movecreator.cpp:233-303): N switchprob
                               attempts per sweep over the particles with a switch type; 0: none */
} sc_run_params;

typedef struct {
    long sweeps;
    long moves;              /* attempted single-particle moves */
    long acc_trans, rej_trans, acc_rot, rej_rot;
    long acc_vol, rej_vol, vol_constrained;   /* vol_constrained: proposals outside the cell-grid range */
    long acc_chain, rej_chain;
    long pairs_tested;       /* candidate pairs scanned (old + new configuration) */
    long pairs_evaluated;    /* pairs that passed the cutoff prefilter */
    double energy;           /* running total energy */
    double energy_check;     /* last exact total energy (check_every) */
    double max_drift;        /* max |running - exact| seen */
    double seconds;          /* device time of the loop (CUDA events on the context's stream) */
    double phase_seconds;    /* device time inside the move kernels (time_phases = 1) */
    long phase_launches;     /* move-kernel launches */
    long launches;           /* all kernels this call launched */
    /* delayed acceptance (delayed = 1) */
    long da_stage1_rejected; /* moves rejected by the surrogate stage (no exact energy evaluated) */
    long da_stage2_tried;    /* moves that reached the exact stage */
    long da_stage2_rejected;
    double da_err_rms;       /* rms of dE - dEs over the moves that reached the exact stage */
    double da_err_mean;      /* mean of dE - dEs over the same moves */
    /* grand-canonical moves (grand_every > 0), all species together */
    long acc_insert, rej_insert, acc_delete, rej_delete;
    long particles;          /* particle count after the call */
    long acc_switch, rej_switch;   /* type switch moves (switchprob > 0) */
} sc_run_stats;

/* Record of one grand-canonical species (Statistics::grand, scOOP/structures/statistics.h;
 * printed by Updater::simulate, updater.cpp:358-373), summed over every run of the context. */
typedef struct {
    int mol_type;            /* molecule type (order of [Molecules]) */
    int type;                /* its particle type */
    int count;               /* molecules of it now */
    int pad_;
    double activity;         /* top.init ACTIVITY */
    double chem_pot;         /* log(activity Nav 1e-24) (inicializer.cpp:1094) */
    long steps;              /* muVtSteps: moves that drew this species */
    long ins_acc, ins_rej, del_acc, del_rej;
    double average_particles;   /* muVtAverageParticles / muVtSteps: mean count after its moves */
} sc_grand_stats;

const char* sc_last_error(void);
const char* sc_version(void);

/* --- set-up: the reference's inputs --------------------------------------------------- */
/* Reads options / top.init / config.init (Sim::readOptions sim.h:123-406,
 * Inicializer::initTop inicializer.cpp:16-58, Inicializer::initConfig :89-298) and
 * derives the interaction table (Topo::genParamPairs topo.cpp:5-153) and the patch
 * vectors (Conf::partVecInit Conf.cpp:97-102).  No device memory is touched until the
 * first energy or move call. */
int sc_open(const char* options_path, const char* top_path, const char* config_path, sc_context** out);
int sc_open_text(const char* options, const char* top, const char* config, sc_context** out);
int sc_close(sc_context* ctx);
int sc_set_device(sc_context* ctx, int device);

/* --- state ------------------------------------------------------------------------------ */
int sc_num_particles(const sc_context* ctx, int* n);
int sc_get_box(sc_context* ctx, double box[3]);
int sc_set_box(sc_context* ctx, const double box[3]);
int sc_cutoff(const sc_context* ctx, double* sqmaxcut, double* maxcut);
int sc_get_pair_param(const sc_context* ctx, int type1, int type2, sc_pair_param* out);
int sc_get_particles(sc_context* ctx, int first, int count, sc_particle* out);
int sc_set_particles(sc_context* ctx, int first, int count, const sc_particle* in);
/* Conf::draw (scOOP/structures/Conf.h:388-425): the config.last text format. */
int sc_write_config(sc_context* ctx, const char* path);

/* --- energies: the TotalE interface ------------------------------------------------------ */
/* TotalE::p2p (totalenergycalculator.h:200-203): PairE(i, j, conlist(i)). */
int sc_pair_energy(sc_context* ctx, int i, int j, double* e);
/* Batched PairE with branch verdicts (bit 0 evaluated, 1 repulsive, 2 attractive branch,
 * 3 far, 8+ intersections) and the closest segment distance^2 (-1 if not evaluated). */
int sc_pair_energies(sc_context* ctx, int npairs, const int* i, const int* j, double* e, unsigned* verdict,
                     double* dist_sq);
/* TotalEMatrix::oneToAll / oneToAllTrial (totalenergycalculator.h:355-415): energy of
 * each target with every other particle. */
int sc_one_to_all(sc_context* ctx, int ntargets, const int* targets, double* e);
/* No counterpart in the reference.  The same energies as sc_one_to_all, for callers
 * that must not allocate device memory: code running while another allocator (for
 * instance a framework's caching allocator) holds all free device memory, so that a
 * cudaMalloc would fail, and latency-critical loops in which a cudaMalloc / cudaFree
 * would synchronise the device.  Targets and results are staged in a fixed array
 * inside the library (SC_NOALLOC_MAX_TARGETS entries, 192 KiB on every GPU that
 * loads the library, held until the process exits); this call allocates nothing.
 *   - At most SC_NOALLOC_MAX_TARGETS targets per call (else SC_ERR_RANGE).
 *   - The context's particle state must already be on the device: make one
 *     allocating call (e.g. sc_one_to_all) after opening or changing it, else
 *     SC_ERR_STATE.
 *   - The array is committed on a device by the first allocating call of any context
 *     there (the lookup of its device address loads the module that holds it), not by
 *     this call: even the first no-alloc call on a device allocates nothing.
 *   - The call runs with the context's device current and gives the caller's current
 *     device back before it returns.
 *   - All calls share the array: calls that overlap on the GPU (other host threads,
 *     other contexts' streams) race; serialise them. */
#define SC_NOALLOC_MAX_TARGETS 16384
int sc_one_to_all_noalloc(sc_context* ctx, int ntargets, const int* targets, double* e);
/* TotalEMatrix::allToAll (totalenergycalculator.h:334-353, 502-521). */
int sc_all_to_all(sc_context* ctx, double* e);
/* Updater::alignmentOrder (scOOP/mc/updater.cpp:466-481): sum of axis dot products over pairs
 * whose centres are closer than 1.5 (the second column of energy.dat). */
int sc_alignment_order(sc_context* ctx, double* order);
/* No counterpart in the reference (its analysis reports the pair alignment above): the
 * nematic order parameter S2, the largest eigenvalue of Q = <3/2 u u^T - 1/2 I> over the
 * axes u of the spherocylinders (spheres excluded), and the director (its unit eigenvector,
 * may be NULL).  1 for a perfectly aligned phase, about 0 for an isotropic one; 0 when the
 * system holds no spherocylinder. */
int sc_nematic_order(sc_context* ctx, double* s2, double director[3]);
/* TotalEMatrix::mol2othersTrial (totalenergycalculator.h:453-499). */
int sc_mol_to_others(sc_context* ctx, int first, int size, double* e);
/* The energy half of MoveCreator::partDisplace / partRotate (movecreator.cpp:947-1028):
 * old energy of the target, and its energy after displacing it by dr (box fractions) or
 * after Particle::pscRotate(angle, axis, sign) (particle.h:182-272) followed by the
 * re-orthogonalisation of patchdir[0].  The state is unchanged until sc_accept_trial(). */
int sc_trial_displace(sc_context* ctx, int target, const double dr[3], double* e_old, double* e_new);
int sc_trial_rotate(sc_context* ctx, int target, double angle, const double axis[3], int positive, double* e_old,
                    double* e_new, sc_particle* trial_state);
int sc_accept_trial(sc_context* ctx);
/* Isotropic volume trial (movecreator.cpp:390-421): allToAllTrial with every box edge + psch. */
int sc_trial_volume(sc_context* ctx, double psch, double* e_new);

/* --- the move loop: Updater::simulate (scOOP/mc/updater.cpp:45-389) --------------------- */
int sc_default_run(const sc_context* ctx, sc_run_params* p);
/* Runs p->nsweeps sweeps on the device; stats->sweeps is the number run (fewer when a
 * Wang-Landau run converged, as the reference's loop stops there, updater.cpp:255-265). */
int sc_simulate(sc_context* ctx, const sc_run_params* p, sc_run_stats* stats);
/* Grand-canonical species (molecule types with a top.init ACTIVITY; options nGrandCanon must
 * be > 0 then, and the species single particles listed after every chain type): *count gets
 * their number.  sc_grand_stats_get fills species k's record (0 <= k < count).  With
 * grand_every > 0 the particle count changes on the device: sc_num_particles and
 * sc_get_particles see the new vector after the call, which keeps the reference's order
 * (an insertion at the end of its species' block, a deletion closing its slot). */
int sc_grand_species(const sc_context* ctx, int* count);
int sc_grand_stats_get(const sc_context* ctx, int k, sc_grand_stats* out);
/* top.last (main.cpp:313-331): the context's top.init text up to and including its [System]
 * line, then "name count" for every molecule type with the current counts. */
int sc_write_top_last(sc_context* ctx, const char* path);

/* --- equilibration: adaptation of the maximum steps (Updater::simulate's adjustment block,
 * scOOP/mc/updater.cpp:238-253, with optimizeStep / optimizeRot, updater.cpp:395-464, and
 * the equilibrate-then-produce sequence of main.cpp:270-297) ------------------------------ */
typedef struct {
    double trans[40];          /* maximum displacement per particle type (full length, as transmx) */
    double rot_cos[40];        /* the reference's rotation record per type: cos of the maximum angle,
                                  adapted by optimizeRot; as in the reference (whose rotations read
                                  Disp::angle) the moves keep the options' rotation angle */
    double chain_trans[8];     /* chain displacement per molecule type */
    double chain_rot_cos[8];
    double edge;               /* box edge change range (as edge_mx) */
    long adjustments;          /* sc_adjust_steps applications so far */
    long acc_trans[40], rej_trans[40], acc_rot[40], rej_rot[40];       /* the counts of the last run */
    long acc_chain_trans[8], rej_chain_trans[8], acc_chain_rot[8], rej_chain_rot[8];
    long acc_edge, rej_edge;
} sc_step_sizes;
int sc_get_step_sizes(sc_context* ctx, sc_step_sizes* out);
/* One adjustment on the last run's acceptance counts: optimizeStep on the displacement of every
 * particle type and chain molecule type that moved (upper bound 1.5), optimizeRot on their
 * rotation records (5.0, 0.01) and optimizeStep on the box edge (1.0).  Later runs displace
 * by the adapted per-type steps (scaled as the run's transmx / chainmmx scale the options'
 * values) and sc_default_run returns the adapted edge range. */
int sc_adjust_steps(sc_context* ctx);
/* main.cpp:270-287: nequil/2 sweeps with an adjustment every `adjust` sweeps (none with
 * adjust = 0), then nequil/2 sweeps without; stats sums both.  Write config.eq afterwards with
 * sc_write_config (the same format). */
int sc_equilibrate(sc_context* ctx, const sc_run_params* p, long nequil, long adjust, sc_run_stats* stats);

/* No counterpart in the reference (its loop has no launch shapes to choose).  Times every
 * candidate launch shape of the move kernel for p's mode (plain or delayed) on the context's
 * current state, `sweeps` sweeps each after two warm-up sweeps: cell reach 1, 2, 3 (cells
 * maxcut/reach wide: how many cells move at once and how many neighbours each stages) times
 * kernel variants {colour-phase launches, dataflow sweep} x {lowest latency per move, more
 * CTAs per SM}, plus paired passes and the warp-per-cell sweep for plain moves.  The state is
 * restored before every
 * candidate and at the end (the next run recomputes the exact energy).  *best = *p with the
 * fastest stencil and variant, which later runs with variant = -1 use.  rates (may be NULL,
 * room for 24) gets each candidate's moves/s, *ncand (may be NULL) their number.  Not with
 * Wang-Landau weights (SC_ERR_UNSUPPORTED: the tuning sweeps would change them). */
int sc_tune(sc_context* ctx, const sc_run_params* p, int sweeps, sc_run_params* best, double* rates, int* ncand);

/* No counterpart in the reference: the move kernels' candidate screens, exposed so that
 * they can be checked against the reference's prefilter (PairE::operator(), paire.h:1209-1215:
 * r^2 > sqmaxcut and no bond -> energy 0).  For every target (targets[0..ntargets), or every
 * particle when targets is NULL) and every other particle j, stage A is the FP32 candidate
 * screen the kernels stage neighbours with (wrapped FP32 box fractions against (maxcut +
 * margin)^2) and stage B their FP32 exact-zero screen (segment or point-segment distance
 * beyond every branch's cut-off).  The pairs that pass stage A go to i[], j[] (in no
 * particular order) with stage_b[k] = 1 when stage B keeps the pair; *count gets their
 * number, SC_ERR_RANGE when it exceeds cap (nothing beyond cap is written).  The kernels
 * evaluate bonded partners whatever these screens say. */
int sc_screen_survivors(sc_context* ctx, int ntargets, const int* targets, long cap, int* i, int* j,
                        unsigned char* stage_b, long* count);

/* No counterpart in the reference.  FP64 rates of `device`, measured by the library's own
 * probe kernels (the denominators of the move kernel's FP64 roofline): separate DMUL + DADD
 * instructions per second with every SM full of warps; the same with one active lane per
 * warp (per-lane rate; equal to the full rate / 32 when an FP64 warp instruction costs the
 * same whatever its active lanes); DFMA FLOP/s (2 per FMA); the dependent latency of one
 * FP64 operation in cycles.  Any output may be NULL.  Allocates and frees a small buffer. */
int sc_fp64_rates(int device, double* dmul_dadd_per_s, double* one_lane_per_s, double* fma_flops,
                  double* latency_cycles);

/* --- Wang-Landau flat-histogram sampling --------------------------------------------------
 * WangLandau (scOOP/mc/wanglandau.h:16-690, wanglandau.cpp): with options wlm > 0 every move
 * is biased by the weights of one or two order parameters, the visited bin's weight drops
 * by alpha after every move, and every 1000 sweeps alpha is halved once the histogram is
 * flat (the run ends when alpha falls below 1e-8).  Supported order parameters (options wlm):
 * 1 z of particle 0 relative to the system's volume-weighted centre, 3 z component of
 * particle 0's axis, 4 xy distance of particles 0 and 1, 7 particles of type wlmtype within
 * distance 6 of particle 0, 8 / 9 box length in x / y; the mesh-hole and pore orders 2, 5, 6
 * are SC_ERR_UNSUPPORTED, and so is order 7 with chain moves of chains that hold particles
 * of type wlmtype.
 * sc_simulate applies the bias once weights are loaded; with wlm > 0 and none loaded it
 * returns SC_ERR_STATE (the reference stops without wl.dat).  sc_open loads wl.dat from
 * the options file's directory when it exists.  Wang-Landau weights in a replica batch
 * need exchange_every = 0 (walkers, see sc_wl_share). */
typedef struct {
    int dim;                 /* order parameters (1 or 2) */
    int wlm[2];
    int length[2];           /* bins; length[1] = 0 for one order parameter, as the reference */
    int converged;           /* a flatness check found alpha below 1e-8: the run stops there */
    double minorder[2], dorder[2];
    double alpha;
    long currorder[2];       /* current bins */
    long updates;            /* alpha halvings so far */
    double syscm[3];         /* system centre (box fractions) the order 1 bin is measured from */
} sc_wl_info;
/* WangLandau::initCalc + init (wanglandau.cpp:49-137, 168-299): reads the weights file (alpha,
 * then "order weight hist" or "order0 order1 weight hist" lines) and computes the starting
 * bins; a starting bin outside the file's range is SC_ERR_RANGE. */
int sc_wl_load(sc_context* ctx, const char* path);
int sc_wl_load_text(sc_context* ctx, const char* text);
int sc_wl_get_info(sc_context* ctx, sc_wl_info* out);
/* Multiple walkers (the reference's MPI walkers sharing weights and histogram through
 * shared-memory windows, wanglandau.cpp:184-218): walkers[1..n-1] drop their own weights and
 * update walkers[0]'s, which runs the flatness checks.  All need the same order parameters
 * and bins and one device; run them together with sc_replicas_run (exchange_every = 0),
 * where every walker's moves of a sweep update the shared histogram before the check. */
int sc_wl_share(sc_context* const* walkers, int n);
/* Current weights and histogram, length[0] * max(1, length[1]) entries each (either may be NULL). */
int sc_wl_get(sc_context* ctx, double* weights, long* hist);
/* WangLandau::write (wanglandau.cpp:139-166): the weights file format. */
int sc_wl_write(sc_context* ctx, const char* path);
/* WangLandau::endWangLandau (wanglandau.cpp:404-433): shifts 2-D weights by the first bin's
 * (its loop leaves 1-D weights as they are) and writes the file. */
int sc_wl_end(sc_context* ctx, const char* path);

/* --- parallel tempering: replicas moved together ------------------------------------------
 * The reference runs one replica per MPI rank and exchanges temperatures in
 * MoveCreator::replicaExchangeMove (scOOP/mc/movecreator.cpp:552-795).  Here all replicas
 * (contexts on one GPU, any N) are moved by the same kernels in one launch sequence
 * (captured as a CUDA graph), and the exchange is a device step over the replicas'
 * running energies.  ladder[k] groups replicas into independent temperature ladders
 * (NULL: one ladder); members of a ladder must hold the same system (N, types).  The
 * contexts stay owned by the caller and must outlive the replica set. */
typedef struct sc_replicas sc_replicas;
int sc_replicas_create(sc_context* const* systems, int nrep, const double* temperatures, const int* ladder,
                       sc_replicas** out);
/* Runs p->nsweeps sweeps of every replica (p's temper is ignored: each replica keeps its
 * ladder temperature; step sizes come from each replica's options unless p sets them),
 * with an exchange attempt every exchange_every sweeps (0: none).  Outputs per replica
 * (each may be NULL): its current temperature, running energy, and the exchange attempts
 * / acceptances of ladder slot k with slot k+1. */
int sc_replicas_run(sc_replicas* r, const sc_run_params* p, int exchange_every, sc_run_stats* stats,
                    double* temperatures, double* energies, long* exchanges_tried, long* exchanges_accepted);
int sc_replicas_destroy(sc_replicas* r);

/* --- learned pair-energy surrogate and delayed acceptance ------------------------------------
 * No counterpart in the reference.  A small network (16 -> 64 -> 64 -> 64 -> 1, SiLU, BF16
 * weights, FP32 accumulation on the tensor cores) learns, per ordered SC-SC pair closer
 * than the largest patch cut-off, the exact pair energy minus the FP32 WCA of the segment
 * distance.  With delayed = 1 a move is first tested with the surrogate's energy change
 * dEs and only then with the exact FP64 change dE against exp(-(dE - dEs)/T): the chain
 * samples the exact Boltzmann distribution, and moves the first stage rejects never
 * evaluate an exact pair energy.  A surrogate belongs to the types of the context it was
 * created from and lives on that context's device. */
typedef struct sc_surrogate sc_surrogate;
typedef struct {
    int epochs;
    int batch;              /* rows per step, a multiple of 64 */
    double lr;              /* peak Adam learning rate */
    double lr_final;        /* end of the cosine decay (0: lr / 50) */
    int warmup_steps;       /* linear warm-up */
    int pad_;
    unsigned long long seed;
} sc_train_params;
typedef struct {
    long steps;
    long samples;
    double loss_first;      /* mean squared error of the first step's batch */
    double loss_last;       /* and of the last step's batch */
    double seconds;         /* host wall time of the training call */
} sc_train_stats;
/* capacity: training samples the surrogate can hold (68 bytes each on the device) */
int sc_surrogate_create(sc_context* ctx, unsigned long long seed, long capacity, sc_surrogate** out);
int sc_surrogate_destroy(sc_surrogate* s);
/* Appends the samples of ctx's current configuration (every ordered SC-SC pair within
 * range: features and exact FP64 pair energy - WCA32); *total = samples held. */
int sc_surrogate_collect(sc_surrogate* s, sc_context* ctx, long* total);
int sc_surrogate_num_samples(const sc_surrogate* s, long* n);
/* Mini-batch Adam on the collected samples; loss_per_epoch (may be NULL) gets the last
 * batch's mean squared error of each epoch. */
int sc_surrogate_train(sc_surrogate* s, const sc_train_params* p, double* loss_per_epoch, sc_train_stats* stats);
/* Network error against the exact energies of ctx's current configuration. */
int sc_surrogate_evaluate(sc_surrogate* s, sc_context* ctx, double* rmse, double* mae, double* max_abs, long* npairs);
/* FP32 master weights, 9409 floats: W1[16][64] (row 12 = first-layer bias, rows 13-15
 * unused), W2[64][64], b2[64], W3[64][64], b3[64], W4[64], b4. */
int sc_surrogate_get_weights(sc_surrogate* s, float* theta);
int sc_surrogate_set_weights(sc_surrogate* s, const float* theta);
/* One forward/backward on the tensor cores over n given rows (16 inputs each): gradient of
 * the mean squared error with respect to the 9409 masters, and that error. */
int sc_surrogate_gradient(sc_surrogate* s, int n, const float* inputs, const float* targets, float* grad,
                          double* loss);
/* Network outputs of n given rows (the move kernel's forward). */
int sc_surrogate_predict(sc_surrogate* s, int n, const float* inputs, float* out);
/* The 16 inputs, WCA32 and eligibility (1: SC-SC, not bonded, within range) of ordered pairs
 * (i[k] moved, j[k] neighbour), as the move kernel computes them. */
int sc_pair_features(sc_context* ctx, int npairs, const int* i, const int* j, float* inputs, float* wca,
                     int* eligible);
/* Attaches s (NULL detaches) as the first stage of ctx's delayed-acceptance moves; s must
 * outlive the attachment. */
int sc_set_surrogate(sc_context* ctx, sc_surrogate* s);

#ifdef __cplusplus
}
#endif
#endif /* SC_GB300_H */
