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

/* P(rxg,defg) by the reference's formula, for pinning the table against the reference */
double oracle_mobility_weight(const score_params* p, const double* qr, const double* qd);

#ifdef __cplusplus
}
#endif
#endif
