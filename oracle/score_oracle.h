/*
 * CPU oracle of the recrystallization growth step — TEST INFRASTRUCTURE ONLY.
 *
 * A single-threaded plain-C restatement of SCORE's growth machine in its
 * canonical one-region form (caHdl::solve_RXGROWTH with OMP_NUM_THREADS=1,
 * src/SCORE_Kernel.cpp:6497-6792).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU baseline may call it; the product never links or loads it.
 *
 * Pinning: tests compare this oracle bit for bit against the reference itself
 * (compiled from its own sources by oracle/ref/Makefile, run through
 * oracle/ref/score_ref_driver.cpp) and against the committed golden fixtures in
 * tests/golden/ that the reference produced.  Features the reference lacks
 * (fully periodic boundary, rho0/(1+kt) recovery, incubation times, growable
 * Border list) are "parity unpinned": the oracle is then the only checker.
 */
#ifndef SCORE_ORACLE_H
#define SCORE_ORACLE_H
#include <stdint.h>
#include "../include/score_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_step {
    uint32_t step, n_nuclei;
    double t, dt, dt_used, Xcells, X;
    uint64_t Sv, n_full, n_new;
    double Pmax, rhomax, dXstep;
    uint32_t next_never[2], n_recycled[2];
} oracle_step;

typedef struct oracle_out {
    uint32_t n_steps;
    int status;            /* SCORE_OK or a SCORE_ERR_* code */
    double dt0;            /* dt before the first step */
    double Pmax0;          /* P max after site-saturated nucleation */
    uint32_t n_nuclei;     /* nuclei placed */
    double seconds;        /* wall time of the step loop */
} oracle_out;

/* Runs nucleation + the step loop until the reference's stop rule with x_target
 * (x_target < 0 uses p->xmax) or max_steps steps.  labels (N), rxg_counts (nrxg),
 * defg_counts (ndefg) and trace (trace_cap rows) may be NULL. */
int oracle_run(const score_params* p, const uint32_t* grid, const double* defg_q, const double* defg_rho0, uint32_t ndefg,
               const double* rxg_q, const uint32_t* rxg_site, const double* rxg_tincub, uint32_t nrxg, const double* ptable,
               double x_target, uint32_t max_steps, oracle_step* trace, uint32_t trace_cap, uint32_t* labels,
               uint32_t* rxg_counts, uint32_t* defg_counts, oracle_out* out);

/* The same run in pieces, for timing bounded samples of a long run: create (the
 * solve_RXGROWTH prologue and site-saturated nucleation), advance (the step loop until
 * the stop rule with x_target, or max_steps more steps; out->n_steps and out->seconds
 * cover this call only, trace rows are this call's steps), done (the stop rule holds),
 * finish (labels and counts), destroy.  The input arrays must outlive the handle. */
typedef struct oracle_sim oracle_sim;
oracle_sim* oracle_create(const score_params* p, const uint32_t* grid, const double* defg_q, const double* defg_rho0, uint32_t ndefg,
                          const double* rxg_q, const uint32_t* rxg_site, const double* rxg_tincub, uint32_t nrxg,
                          const double* ptable);
int oracle_advance(oracle_sim* o, double x_target, uint32_t max_steps, oracle_step* trace, uint32_t trace_cap, oracle_out* out);
int oracle_done(const oracle_sim* o, double x_target);
void oracle_finish(const oracle_sim* o, uint32_t* labels, uint32_t* rxg_counts, uint32_t* defg_counts);
void oracle_destroy(oracle_sim* o);
double oracle_time(const oracle_sim* o);   /* t after the last step */

/* The grain-evolution log of a run (params n_logpoints / logpoint_x / rxarea_threshold): per snapshot the
 * time before the logged step, X after it, its step index and 32-bit Sv, every grain's cell count
 * (ndefg + nrxg, deformed first) and the RX area profile (2 nz: rx cells, the rest, per z slice). */
uint32_t oracle_log_count(const oracle_sim* o);
int oracle_log_get(const oracle_sim* o, uint32_t i, double* t, double* X, uint32_t* step, uint32_t* sv, uint32_t* counts,
                   uint32_t* area);

/* Ensemble post-processing of grain-evolution logs (SCORE_SolitaryUnitAveraging.cpp). */
typedef struct oracle_evo {
    uint32_t ndefg, nrxg, nsnap;
    const double* t;                /* nsnap snapshot times */
    const uint32_t* counts;         /* nsnap x (ndefg + nrxg) */
    const uint32_t* final_counts;   /* ndefg + nrxg at the end of the run */
    double tsimend, nboxvol;        /* end time of the run, cells of the domain */
    const uint32_t* grain_class;    /* ndefg + nrxg orientation classes (macrotexture), or NULL */
} oracle_evo;
double oracle_interp_count(const oracle_evo* e, uint32_t id, double when);
void oracle_rediscr_kinetics(const oracle_evo* doms, uint32_t ndom, uint32_t nslots, double* t_out, double* vol_out,
                             double* boxvol_out);
void oracle_rediscr_macrotexture(const oracle_evo* doms, uint32_t ndom, uint32_t nslots, uint32_t nclass, double* t_out,
                                 double* vol_out);

/* Percolation of the recrystallized and infected cells (SCORE_PercAnalyzer.cpp, log_PERCOLATION):
 * binarize (grid value >= ndefg), then clusters (see score_oracle.c) with labels (N, 0 = none), their
 * count, the largest, the spanning axes (bit 0 x, 1 y, 2 z) and the sizes ascending. */
void oracle_binarize(const oracle_sim* o, uint8_t* bin);
int oracle_percolation(const uint8_t* bin, uint32_t nx, uint32_t ny, uint32_t nz, int reference_scan, uint32_t* labels,
                       uint32_t* n_clusters, uint32_t* largest, int* percolates, uint32_t* spans, uint32_t* sizes);

/* P(rxg,defg) by the reference's formula, for pinning the table against the reference */
double oracle_mobility_weight(const score_params* p, const double* qr, const double* qd);

#ifdef __cplusplus
}
#endif
#endif
