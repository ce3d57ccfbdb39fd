/*
 * score_gb300 — C ABI of the GB300-native recrystallization (RX) growth step.
 *
 * This boundary replaces the C++ member-function interface that SCORE's growth
 * machine calls inside one OpenMP region (caHdl::solve_RXGROWTH,
 * src/SCORE_Kernel.cpp:6497-6792).  Plain C types only; every function returns
 * an int status (SCORE_OK = 0, negative on error) and never aborts.  Inputs are
 * HOST buffers that the library copies; the context owns all device memory.
 * One context = one domain = one CUDA stream; single-threaded caller.
 *
 * Sequence (mirrors SIMULATE_myCAs, src/SCORE_Kernel.cpp:1693-1756):
 *   score_uds_read -> score_create -> score_load_domain -> score_place_nuclei
 *   -> score_step ... (or score_run_until) -> score_export_labels -> score_destroy
 */
#ifndef SCORE_GB300_H
#define SCORE_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCORE_ABI_VERSION 4

/* status codes */
#define SCORE_OK                     0
#define SCORE_ERR_ARG               -1  /* bad argument / inconsistent sizes */
#define SCORE_ERR_CUDA              -2  /* CUDA runtime error (message in score_last_error) */
#define SCORE_ERR_NOMEM             -3  /* device or host allocation failed */
#define SCORE_ERR_CAPACITY          -4  /* a front list would exceed its device capacity */
#define SCORE_ERR_BORDER_CAPACITY   -5  /* Border list exceeded 2(xy+xz+yz); the reference writes out of bounds here */
#define SCORE_ERR_TIMEOUT           -6  /* a bounded device wait gave up (error flag set by a kernel) */
#define SCORE_ERR_STATE             -7  /* call out of sequence */
#define SCORE_ERR_IO                -8  /* .uds file missing or malformed */
#define SCORE_ERR_KEYLIMIT          -9  /* more infection attempts in one step than the 32-bit claim key can order */
#define SCORE_ERR_NOT_BUILT        -10  /* CUDA path unavailable (no device) */
#define SCORE_ERR_SCRATCH_LIMIT    -11  /* input larger than a no-allocation entry point's static scratch */

#define SCORE_MAX_TABLE 256        /* max rows of the time tables (annealing, drag) and X logpoint lists */

/* mobility models, src/SCORE_Defs_Functionality.h:280-281 (values as read from "MobilityModel") */
#define SCORE_MOBILITY_SEBALD_GOTTSTEIN 1
#define SCORE_MOBILITY_ROLLETT_HOLM     2
/* recovery models, "RecoveryConsider" 0..3; SCORE_RECOVERY_HYPERBOLIC is this library's rho0/(1+k t) law */
#define SCORE_RECOVERY_NONE             0
#define SCORE_RECOVERY_NES_VACCOREDIFF  1
#define SCORE_RECOVERY_NES_SOLUTEDRAG   2
#define SCORE_RECOVERY_MICHALAKPAXTON   3
#define SCORE_RECOVERY_HYPERBOLIC      10
/* Zener drag, "ZenerConsider" 0..2 */
#define SCORE_ZENER_NONE     0
#define SCORE_ZENER_CONSTANT 1
#define SCORE_ZENER_TIMEDEP  2
/* boundary handling of the domain */
#define SCORE_BOUNDARY_REFERENCE 0  /* x,y periodic, z open: SCORE_Kernel.cpp:4362-4377 */
#define SCORE_BOUNDARY_PERIODIC  1  /* x,y,z periodic */
/* fill arithmetic */
#define SCORE_PRECISION_FP64        0  /* bit-exact with the reference */
#define SCORE_PRECISION_FP32_KAHAN  1  /* FP32 fill with Kahan compensation; FP64 dt/P */
/* Border-list overflow policy */
#define SCORE_BORDER_REFERENCE_LIMIT 0 /* fail with SCORE_ERR_BORDER_CAPACITY where the reference overruns */
#define SCORE_BORDER_GROW            1 /* keep appending (slot order unchanged) */

/*
 * Growth parameters in SI units, exactly as the reference holds them after
 * ensembleHdl::init_parameter (src/SCORE_Kernel.cpp:262-960): activation
 * enthalpies already multiplied by echarge, temperatures in K (C + 273.15),
 * cell size in m.  Table rows (annealing schedule, drag) keep the reference's
 * float truncation of "*(ff)" columns (src/SCORE_Io.h:119).
 */
typedef struct score_params {
    uint32_t nx, ny, nz;              /* 3DCAEdgeLengthInCells RD/TD/ND */
    double cellsize;                  /* CellSize [um] * 1e-6 */
    double xmax;                      /* XMAX */
    double tmax;                      /* TIMEMAX [s] */
    uint32_t nmax;                    /* NMAX */
    double maxfillperstep;            /* MAXFILLPERSTEP */
    double initial_cache;             /* InitialCacheSizeRXCells (sets recycle-list caps) */
    double recache;                   /* ReCacheSizeRXCells */
    int32_t defragmentation;          /* OnTheFlyDefragmentation */
    uint32_t n_defrag;                /* HeuristicRXFrontListDefragmentation X points (sorted) */
    double defrag_x[SCORE_MAX_TABLE];
    /* MaterialProperties */
    double G0, dGdt, bZeroCelsius, Tmelt;
    /* BoundaryMobilityModel */
    int32_t mobility_model;
    double LAGBm0, LAGBHact, HAGBm0, HAGBHact, GSm0, GSHact;
    double RH_HAGBm0, RH_HAGBHact, RH_cut, RH_trans, RH_exponent;
    /* RecoveryParameter */
    int32_t recovery_model;
    double VacancyDiffD0, VacancyDiffHact, SoluteDiffD0, SoluteDiffHact, SoluteLsPropFactor, SoluteConcentration;
    double NesAlpha3, NesKappa2, NesC3, NesC4, NesC5;
    double recovery_k;                /* k [1/s] of rho(t)=rho0/(1+k t) (SCORE_RECOVERY_HYPERBOLIC) */
    /* DragParameter / EvoMicrochemistry */
    int32_t zener_model;
    double zener_alpha, zener_gamma;
    uint32_t n_zener;
    double zener_time[SCORE_MAX_TABLE], zener_fr[SCORE_MAX_TABLE];
    /* AnnealingSchedule (K) */
    uint32_t n_schedule;
    double sched_time[SCORE_MAX_TABLE], sched_temp[SCORE_MAX_TABLE];
    /* GB300 build options (no .uds keyword) */
    int32_t boundary;                 /* SCORE_BOUNDARY_* */
    int32_t precision;                /* SCORE_PRECISION_* */
    int32_t border_policy;            /* SCORE_BORDER_* */
    int32_t reserved;
    /* on-the-fly characterization (SCORE_OnTheFlyCharacterization.cpp:635-650) */
    uint32_t n_logpoints;             /* SingleGrainVolOverTime X logpoints (sorted; X read as float, as the reference) */
    double logpoint_x[SCORE_MAX_TABLE];
    uint32_t rxarea_threshold;        /* RXAreaThreshold (GB300Options): rx grain sections of fewer cells are not
                                         counted in the RX area profile; 13 in log_OUTPUT_Diehl */
    uint32_t reserved2;
} score_params;

/* per-step scalars (the master block of solve_RXGROWTH, SCORE_Kernel.cpp:6688-6740) */
typedef struct score_step_stats {
    uint32_t step;        /* steps completed so far */
    uint32_t n_nuclei;    /* nuclei placed before this step (time-dependent nucleation) */
    double t;             /* time after this step [s] (t += dt) */
    double dt;            /* dt for the NEXT step */
    double dt_used;       /* dt this step integrated with */
    double Xcells;        /* fully recrystallized cells */
    double X;             /* Xcells / N */
    uint64_t Sv;          /* ACTIVE front cells updated this step (Inside + Border) */
    uint64_t n_full;      /* cells that completed this step and infected their neighbours */
    uint64_t n_new;       /* cells newly infected this step */
    double Pmax;          /* running max mobility weight P */
    double rhomax;        /* max rho over deformed grains with cells left */
    double dXstep;        /* sum of fill increments (observation; order differs from the reference) */
    uint32_t next_never[2];  /* Inside, Border: slots ever used */
    uint32_t n_recycled[2];  /* Inside, Border: recycle-list lengths this step */
    uint32_t p_misses;       /* mobility weights computed on the host this step */
    uint32_t reserved;
} score_step_stats;

/* one grain-evolution snapshot (loginfo_grainevo_ca, src/SCORE_Kernel.h:642-651) */
typedef struct score_grainevo_info {
    double t;             /* time at the start of the logged step [s]: the reference logs before t += dt */
    double X;             /* recrystallized fraction after the step */
    uint32_t step;        /* steps completed before the logged one */
    uint32_t Sv;          /* front cells updated in the logged step (32-bit, as the reference logs it) */
} score_grainevo_info;

/* library */
int  score_abi_version(void);
const char* score_status_string(int status);

/* .uds input file -> params (ensembleHdl::init_parameter, src/SCORE_Kernel.cpp:1542-1625) */
int  score_params_default(score_params* out);
int  score_uds_read(const char* path, score_params* out);

/* context: caHdl + its caregionMemHdl fronts (src/SCORE_Kernel.h:1008-1347, 1403-1584) */
typedef struct score_ctx score_ctx;
int  score_create(score_ctx** out, const score_params* p, int device);
void score_destroy(score_ctx* ctx);
const char* score_last_error(const score_ctx* ctx);

/*
 * Load one domain (replaces solve_SYNTHESIZE_DEFORMATIONSTRUCTURE + nucleation
 * modelling + solve_REPLACE_CA_STRUCTURE, src/SCORE_Kernel.cpp:6142,6321,6353):
 *   grid       nx*ny*nz deformed-grain ids (x fastest), each < ndefg
 *   defg_quat  ndefg x 4 unit quaternions (q0,q1,q2,q3), defg_rho0 ndefg [1/m^2]
 *   rxg_quat   nrxg x 4, rxg_site nrxg linear sites x+y*nx+z*nx*ny, rxg_tincub nrxg [s] (NULL = all 0)
 *   ptable     optional nrxg*ndefg mobility weights P(rxg,defg) (row = rxg); NULL = computed on the
 *              host in FP64 on first use (caregionMemHdl::reg_calc_mobilityweight, SCORE_Kernel.cpp:2460)
 */
int  score_load_domain(score_ctx* ctx, const uint32_t* grid, const double* defg_quat, const double* defg_rho0,
                       uint32_t ndefg, const double* rxg_quat, const uint32_t* rxg_site, const double* rxg_tincub,
                       uint32_t nrxg, const double* ptable);
/* A context may load again: with the same ndefg/nrxg it reuses its device buffers. */

/* Return the loaded domain to its just-loaded state without any host copy
 * (the device keeps the loaded grid): the start of a fresh solve_RXGROWTH. */
int  score_restart(score_ctx* ctx);

/* site-saturated placement of every nucleus with tincub <= t, in rxg order
 * (caHdl::ompshar_sim_myCA_sitesaturatedNucleation, src/SCORE_GrowthMachine.cpp:50-189) */
int  score_place_nuclei(score_ctx* ctx, uint32_t* n_placed);

/* one growth step: grow -> infect -> reduce -> t+=dt -> physics -> dt
 * (loop body of solve_RXGROWTH, src/SCORE_Kernel.cpp:6617-6743) */
int  score_step(score_ctx* ctx, score_step_stats* out);

/* whole step loop until the reference's stop rule (SCORE_Kernel.cpp:6619):
 * Xcells>=N || X>x_target || step>NMAX || t>t_end || t>TIMEMAX.  x_target<0 uses params.xmax.
 * trace (may be NULL) receives up to trace_cap rows; *n_steps the number of steps run. */
int  score_run_until(score_ctx* ctx, double x_target, score_step_stats* trace, uint32_t trace_cap, uint32_t* n_steps);

/* current scalars (step, t, dt, X, ...) without advancing */
int  score_get_stats(score_ctx* ctx, score_step_stats* out);

/* final grain labels by the clarify rule (ompcrit_clarify_status_infectedcells,
 * src/SCORE_Io_Characterization.cpp:925-1000): deformed id, or ndefg+rxg for
 * recrystallized cells and front cells with fill >= 0.5 */
int  score_export_labels(score_ctx* ctx, uint32_t* labels);

/* per-grain cell counts (caHdl::synchronize_*_counts, SCORE_Kernel.cpp:5983-6028) */
int  score_grain_counts(score_ctx* ctx, uint32_t* rxg_counts, uint32_t* defg_counts);

/* device-side timing since the last load/restart (CUDA events on the context's
 * stream): kernel-only ms per phase, ms of the dominant (grow) kernel, its
 * launches, the algorithmic bytes those launches moved, and run_ms = event time
 * from the start of the restart/reset to the end of the last score_run_until */
/* Device phase times (total, grow, claim, commit, fill) and the algorithmic bytes are sums over
 * the TIMED steps: every timing_every-th step of a run (score_tune), timed_steps of them; the
 * steps in between run without phase events.  Host times and counts cover every step. */
typedef struct score_timing {
    double total_ms;        /* device time of the step kernels */
    double grow_ms;         /* the fill update and the FullRX / recycle lists (k_grow_fill, k_grow_lists) */
    double claim_ms;        /* the infection attempts (k_claim) */
    double commit_ms;       /* resolve, commit (new cells, weights) and step end */
    double host_ms;         /* host wall time inside the step calls, the wait included */
    uint64_t grow_launches; /* steps (every step launches the grow kernels once) */
    double grow_bytes;      /* algorithmic bytes of the timed grow launches */
    double step_bytes;      /* algorithmic bytes of all kernels of the timed steps */
    uint64_t kernel_launches;  /* kernels launched by this context since creation */
    double run_ms;          /* device span of the last restart .. score_run_until */
    double fill_ms;         /* the fill-update kernels alone (part of grow_ms) */
    double wait_ms;         /* host time blocked on the step's stream synchronization */
    double weights_ms;      /* host time computing requested mobility weights (libm FP64) */
    double pre_ms;          /* host time before the launch (nucleation, arguments) */
    double post_ms;         /* host wall time after the wait (mailboxes, weights, physics) */
    uint64_t timed_steps;   /* steps whose device phases were timed */
} score_timing;
int  score_get_timing(score_ctx* ctx, score_timing* out);

/*
 * Launch configuration of the step kernels.  Results do not depend on it (every
 * compaction keeps slot order, every claim is decided by its ordinal); only speed does.
 */
typedef struct score_tune {
    int32_t items;                 /* grow tile = 256 * items front slots: 4, 8 or 16 */
    int32_t fill_blocks_per_sm;    /* k_grow_fill grid = SMs * this */
    int32_t claim_blocks_per_sm;   /* k_claim grid */
    int32_t commit_blocks_per_sm;  /* k_resolve / k_commit grid */
    int32_t use_graph;             /* 1: each step replays one captured CUDA graph */
    int32_t spec_holes_pct;        /* k_grow_fill loads each slot's fill data together with its
                                      infector byte while the last step's INACTIVE share of the
                                      scanned slots was at most this percentage (0 never, 100
                                      always; default 30); otherwise only for ACTIVE slots,
                                      after the byte */
    int32_t timing_every;          /* device phase events on every k-th step of a run (1 every
                                      step, 0 never; default 8): events cost device time */
    uint32_t steps;                /* autotuner: steps it ran */
    double fill_ns_per_slot;       /* autotuner: best grow time per front slot [ns] */
    double claim_ns_per_cell;      /* autotuner: best claim time per full cell [ns] */
    double commit_ns_per_cell;     /* autotuner: best resolve+commit time per full cell [ns] */
} score_tune;
int  score_get_tune(score_ctx* ctx, score_tune* out);
int  score_set_tune(score_ctx* ctx, const score_tune* t);
/* Restart, place nuclei, run up to max_steps steps (0: to x_target, < 0: XMAX) cycling
 * candidate configurations, keep the fastest per kernel group, then restart and place
 * the nuclei again: the context is ready for score_run_until. */
int  score_autotune(score_ctx* ctx, double x_target, uint32_t max_steps, score_tune* out);

/*
 * Batched ensemble: many independent domains (own sizes, grains, nuclei, parameters;
 * one precision) stepped together.  The domains form groups of about equal cell count
 * (two from 64 domains on), each stepped concurrently on its own stream; within a group
 * each step is one sequence of kernels over its running domains, replayed as one CUDA
 * graph, and a domain that meets its stop rule leaves the launches.  Mirrors the reference's ensemble of solitary units that its
 * ranks step one after another (SCORE_Kernel.cpp:1640-1756).  Domain d of a batch
 * accepts the single-domain functions' arguments.  The domains of all live contexts
 * and batches of one device share 64 argument slots: a batch holds at most 64 domains,
 * and score_create / score_batch_create return SCORE_ERR_CAPACITY when the device's
 * slots are taken.
 */
typedef struct score_batch score_batch;
int  score_batch_create(score_batch** out, const score_params* params, uint32_t ndomains, int device);
void score_batch_destroy(score_batch* b);
const char* score_batch_last_error(const score_batch* b);
int  score_batch_load_domain(score_batch* b, uint32_t d, const uint32_t* grid, const double* defg_quat,
                             const double* defg_rho0, uint32_t ndefg, const double* rxg_quat,
                             const uint32_t* rxg_site, const double* rxg_tincub, uint32_t nrxg, const double* ptable);
int  score_batch_restart(score_batch* b);
int  score_batch_place_nuclei(score_batch* b);
/* step all domains until each meets its stop rule (x_target < 0: its XMAX) or max_steps (0: no limit) */
int  score_batch_run_until(score_batch* b, double x_target, uint32_t max_steps, uint32_t* steps_done);
int  score_batch_get_stats(score_batch* b, uint32_t d, score_step_stats* out);
/* per-step stats of domain d in the last score_batch_run_until */
int  score_batch_trace(score_batch* b, uint32_t d, score_step_stats* trace, uint32_t cap, uint32_t* n_steps);
int  score_batch_export_labels(score_batch* b, uint32_t d, uint32_t* labels);
int  score_batch_grain_counts(score_batch* b, uint32_t d, uint32_t* rxg_counts, uint32_t* defg_counts);
int  score_batch_get_timing(score_batch* b, score_timing* out);
int  score_batch_get_tune(score_batch* b, score_tune* out);
int  score_batch_set_tune(score_batch* b, const score_tune* t);
int  score_batch_autotune(score_batch* b, double x_target, uint32_t max_steps, score_tune* out);

/*
 * On-the-fly characterization (caHdl::log_OUTPUT_Diehl, src/SCORE_OnTheFlyCharacterization.cpp:635-650).
 * After a step whose X reaches the next SingleGrainVolOverTime logpoint (params n_logpoints /
 * logpoint_x; at most one snapshot per step, as the reference) the device records every grain's
 * cell count (log_grainevo, :478-531: deformed grains, then rx grains) and the RX area profile
 * (log_rxareaprofile(threshold), :274-384: per z slice the cells of the rx grains whose section has
 * at least params rxarea_threshold cells, then the slice's other cells; labels by the clarify rule).
 * The log belongs to the last run (score_restart / score_load_domain clear it).
 *   counts  ndefg + nrxg values, or NULL      rxarea  2 nz values (rx, rest per slice), or NULL
 */
int  score_grainevo_count(score_ctx* c, uint32_t* n);
int  score_grainevo(score_ctx* c, uint32_t i, score_grainevo_info* info, uint32_t* counts, uint32_t* rxarea);
int  score_batch_grainevo_count(score_batch* b, uint32_t d, uint32_t* n);
int  score_batch_grainevo(score_batch* b, uint32_t d, uint32_t i, score_grainevo_info* info, uint32_t* counts,
                          uint32_t* rxarea);

/*
 * Ensemble post-processing on the device (ensembleHdl::postprocess_*, src/SCORE_SolitaryUnitAveraging.cpp)
 * over the grain-evolution logs of a batch's domains (or of one context, an ensemble of one).
 * Time slots: t_n = (n + 1) tmax / (nslots - 1), n < nslots, tmax the latest end time of the domains
 * (postprocess_init + postprocess_initrediscrtimes, :50-80, 510-540).  A grain's volume at t_n is
 * caHdl::get_interpCellCount (:1304-1365): its final count at or after the end of its run, else
 * linear between the snapshots around t_n.  Sums run in the reference's order, so FP64 results are
 * the reference's bits.
 *   kinetics   rxvol[n] = sum over domains of (cells - interpolated deformed volume) (:546-670);
 *              boxvol = cells of all domains; X(t_n) = rxvol[n] / boxvol
 *   texture    vol[n nclass + k] = interpolated volume of the grains of orientation class k, deformed
 *              and rx (:673-804); grain_class holds every domain's ndefg + nrxg classes in domain
 *              order, each < nclass <= 32
 *   grain sizes  every domain's rx grains' final cell counts, in domain order (the final grain-size
 *              distribution's volumes, :808-905)
 */
int  score_rediscr_kinetics(score_ctx* c, uint32_t nslots, double* t_out, double* rxvol_out, double* boxvol_out);
int  score_batch_rediscr_kinetics(score_batch* b, uint32_t nslots, double* t_out, double* rxvol_out, double* boxvol_out);
int  score_batch_rediscr_texture(score_batch* b, uint32_t nslots, const uint32_t* grain_class, uint32_t nclass,
                                 double* t_out, double* vol_out);
int  score_batch_final_grain_sizes(score_batch* b, uint32_t* rx_cells);

/*
 * Percolation analysis of the recrystallized and infected cells on the device (caHdl::log_PERCOLATION,
 * src/SCORE_OnTheFlyCharacterization.cpp:777-875, and percAnalyzer, src/SCORE_PercAnalyzer.cpp), between
 * steps.  Cells with grid value >= ndefg (binarize_partiallyrxed_microstructure, :732-774) form clusters
 * over the six face neighbours, not periodic; the cell at the origin never joins one (the reference labels
 * clusters with cell indices and reads label 0 as "not recrystallized").  Clusters are numbered 1..n in
 * the order of their first cell (compactify, :334-390).
 *   SCORE_PERC_REFERENCE  the reference's clusters: its Hoshen-Kopelman scan links a cell with all three
 *                         lower neighbours present to the lower y and z ones only (:218-225), which can
 *                         split a true cluster (its checkLabeling then reports the split)
 *   SCORE_PERC_CONNECTED  the true 6-connected clusters
 * out: count, largest, P_L = largest / N, percolates (a cluster touches both faces of an axis, :500-615)
 * with the axes in `spans`; sizes: the cluster sizes ascending (determine_clustersize_distr, :617-656),
 * the first sizes_cap of them, or NULL; labels: every cell's cluster (0 = none), N values, or NULL.
 * Reference domains are cubes; any box is accepted here.
 */
#define SCORE_PERC_REFERENCE 0
#define SCORE_PERC_CONNECTED 1
typedef struct score_perc_result {
    uint32_t n_clusters;
    uint32_t largest;
    double PL;
    int32_t percolates;
    uint32_t spans;            /* bit 0: along x, 1: y, 2: z */
} score_perc_result;
int  score_percolation_analyze(score_ctx* c, int mode, score_perc_result* out, uint32_t* sizes, uint32_t sizes_cap, uint32_t* labels);
int  score_batch_percolation_analyze(score_batch* b, uint32_t d, int mode, score_perc_result* out, uint32_t* sizes, uint32_t sizes_cap,
                             uint32_t* labels);

/* FP64 mobility weight P(rxg,defg) on the host, the reference's formula
 * (SCORE_Kernel.cpp:2460-2527, SCORE_Math.cpp:558-622,1067-1130) */
int  score_mobility_weight(const score_params* p, const double* rxg_q, const double* defg_q, double* P);

/*
 * No counterpart in the reference (it evaluates P pair by pair on the host,
 * SCORE_Kernel.cpp:2460-2527).  Device FP64 table of P(rxg, defg) for all
 * nrxg x ndefg pairs and its maximum, for callers that cannot allocate device
 * memory.  cudaMalloc and cudaFree synchronize the whole device and can fail once
 * another allocator (a framework's caching allocator, a fixed per-process budget)
 * holds the memory; a caller that runs beside other streams' work, or inside such
 * a budget, can call this instead of building the table through a context.
 *
 *   d_rxg_quat  device, nrxg x 4 quaternions      d_defg_quat  device, ndefg x 4
 *   d_table     device, nrxg x ndefg doubles (row rxg, column defg), written
 *   d_pmax      device, one double, written with the maximum of the table
 *   stream      cudaStream_t the kernel is launched on (NULL = legacy default stream)
 * Runs on the calling thread's current device and returns after the launch; the
 * results are ready when the stream reaches that point.  Allocates nothing: its
 * only scratch is a static 512 KiB device array with one word per row, so nrxg is
 * at most 65536 (SCORE_ERR_SCRATCH_LIMIT above that, nothing launched).  The
 * scratch holds a completion counter, cleared on the stream (cudaMemsetAsync, no
 * allocation) before every launch.  The first call on a device resolves the
 * scratch address (cudaGetSymbolAddress, which may load the library's device code)
 * and keeps it for the life of the process: a caller that resets the device
 * (cudaDeviceReset) after that first call must not call this entry point again.  A
 * caller that captures streams into graphs makes that first call before it begins
 * a capture.  Calls on the same
 * device share the scratch: calls that overlap in time (two streams, two host
 * threads) race and must be serialized by the caller.  Entries agree with
 * score_mobility_weight to a few ulp (CUDA's acos/cos/exp/pow instead of libm);
 * a pair within a few ulp of the 15-degree or 10-degree threshold can fall into
 * the other class.
 */
int  score_mobility_table_noalloc(const score_params* p, const double* d_rxg_quat, uint32_t nrxg,
                                  const double* d_defg_quat, uint32_t ndefg, double* d_table,
                                  double* d_pmax, void* stream);

/*
 * Deterministic synthetic domain (identical bits on x86-64 and aarch64): periodic
 * Voronoi deformed grains (optionally anisotropic "pancake" metric), uniform or
 * texture-clustered orientations, lognormal or bimodal rho, distinct nucleation
 * sites (uniform or grain-boundary biased), Poisson incubation times.
 */
typedef struct score_gen_params {
    uint32_t nx, ny, nz;
    uint32_t ngrains, nnuclei;
    uint64_t seed;
    double rho_mean, rho_sigma;        /* lognormal: mean and sigma of ln(rho) */
    int32_t rho_mode;                  /* 0 lognormal, 1 bimodal (rho_lo/rho_hi, 50/50) */
    double rho_lo, rho_hi;
    double aspect[3];                  /* Voronoi metric scale per axis (1,1,1 = isotropic) */
    int32_t ori_mode;                  /* 0 uniform, 1 clustered around ncomp components */
    uint32_t ncomp;
    double scatter_deg;                /* Gaussian scatter around components */
    int32_t site_mode;                 /* 0 uniform, 1 grain-boundary biased */
    double gb_fraction;                /* fraction of nuclei forced onto boundary cells (site_mode 1) */
    double nucleation_rate;            /* >0: Poisson incubation times at this rate [1/s]; 0: all 0 */
} score_gen_params;
int  score_gen_default(score_gen_params* out);
int  score_generate_domain(const score_gen_params* g, uint32_t* grid, double* defg_quat, double* defg_rho0,
                           double* rxg_quat, uint32_t* rxg_site, double* rxg_tincub);
/*
 * The same domain with the Voronoi label fill on the device: deformed-structure synthesis on the
 * GPU (the reference synthesizes its deformed structures on the host, src/SCORE_StructureSynthesis.cpp:
 * cuboid voxelizer :466-529, unit-speed CA tessellation :164-345).  Every output is bit for bit
 * score_generate_domain's: the nearest-seed search and its FP64 arithmetic are the host's.  The
 * label grid comes back into the host buffer `grid` (the nuclei placement reads it).
 */
int  score_generate_domain_gpu(const score_gen_params* g, uint32_t* grid, double* defg_quat, double* defg_rho0,
                               double* rxg_quat, uint32_t* rxg_site, double* rxg_tincub, int device);

#ifdef __cplusplus
}
#endif
#endif
