/*
 * CPU oracle of SCORE's recrystallization growth step — TEST INFRASTRUCTURE ONLY
 * (see score_oracle.h).  Sequential, FP64, AoS front lists with the reference's
 * slot allocator, recycle caps and stop rule.  Each function cites the reference
 * code it restates.  Build: gcc -O2 -ffp-contract=off (no FMA contraction, so
 * FP64 results equal the reference's -ffp-contract=off / x86-64 SSE2 build).
 */
#include "score_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define CURRENTLY_INFECTED 4096002000u
#define RHO_RX 1.0e11
#define PI_ 3.1415926535897932384626433832795
#define KB 1.3806488e-23
#define INFINITE_ 1e36
#define RHOMAX_WELLANNEALED 1e8

/* ------------------------------------------------------------------ mobility weight */
/* multiply_quat_degraef, SCORE_Math.cpp:230-239 (P_EIJK = +1) */
static void qmul(const double* p, const double* q, double* r) {
    r[0] = p[0] * q[0] - p[1] * q[1] - p[2] * q[2] - p[3] * q[3];
    r[1] = q[0] * p[1] + p[0] * q[1] + (+1.0 * p[2] * q[3] - 1.0 * p[3] * q[2]);
    r[2] = q[0] * p[2] + p[0] * q[2] + (-1.0 * p[1] * q[3] + 1.0 * p[3] * q[1]);
    r[3] = q[0] * p[3] + p[0] * q[3] + (+1.0 * p[1] * q[2] - 1.0 * p[2] * q[1]);
}

/* the six Grimmer quaternions of SCORE_Math.cpp:581-594 / 1091-1104 */
static void grimmer(const double* p, const double* q, double r0[6][4]) {
    double qm1[4] = {q[0], -1.0 * q[1], -1.0 * q[2], -1.0 * q[3]};
    double r[4];
    qmul(qm1, p, r);
    double a = r[0], b = r[1], c = r[2], d = r[3];
    double fac = 1.0 / sqrt(2.0);
    r0[0][0] = (a + b) * fac; r0[0][1] = (a - b) * fac; r0[0][2] = (c + d) * fac; r0[0][3] = (c - d) * fac;
    r0[1][0] = (a + c) * fac; r0[1][1] = (a - c) * fac; r0[1][2] = (b + d) * fac; r0[1][3] = (b - d) * fac;
    r0[2][0] = (a + d) * fac; r0[2][1] = (a - d) * fac; r0[2][2] = (b + c) * fac; r0[2][3] = (b - c) * fac;
    r0[3][0] = (a + b + c + d) * 0.5; r0[3][1] = (a + b - c - d) * 0.5; r0[3][2] = (a - b + c - d) * 0.5; r0[3][3] = (a - b - c + d) * 0.5;
    r0[4][0] = (a + b + c - d) * 0.5; r0[4][1] = (a + b - c + d) * 0.5; r0[4][2] = (a - b + c + d) * 0.5; r0[4][3] = (a - b - c - d) * 0.5;
    r0[5][0] = a; r0[5][1] = b; r0[5][2] = c; r0[5][3] = d;
}

/* disori_angle_oriquat_cubic_imm, SCORE_Math.cpp:558-622 */
static double disori_angle(const double* p, const double* q) {
    double r0[6][4];
    grimmer(p, q, r0);
    double omega = 0.0;
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 4; j++)
            if (fabs(r0[i][j]) > omega) omega = fabs(r0[i][j]);
    if (omega < (1.0 - 5.0e-16)) return 2.0 * acos(omega);
    return 0.0;
}

/* disori_fromoriquat_cubic_imm, SCORE_Math.cpp:1067-1130 (bubble sort ascending, then reversed) */
static void disori_quat(const double* p, const double* q, double* quat) {
    double r0[6][4];
    grimmer(p, q, r0);
    int mi = 0;
    double mx = 0.0;
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 4; j++)
            if (fabs(r0[i][j]) > mx) { mx = fabs(r0[i][j]); mi = i; }
    double rq[4] = {fabs(r0[mi][0]), fabs(r0[mi][1]), fabs(r0[mi][2]), fabs(r0[mi][3])};
    int last = 2, changed = 1;
    while (last >= 0 && changed) {
        changed = 0;
        for (int k = 0; k <= last; k++)
            if (rq[k] > rq[k + 1]) { double t = rq[k]; rq[k] = rq[k + 1]; rq[k + 1] = t; changed = 1; }
        last--;
    }
    quat[0] = rq[3]; quat[1] = rq[2]; quat[2] = rq[1]; quat[3] = rq[0];
}

/* caregionMemHdl::reg_calc_mobilityweight, SCORE_Kernel.cpp:2460-2527 */
double oracle_mobility_weight(const score_params* prm, const double* q1, const double* q2) {
    double theta = disori_angle(q1, q2);
    const double lagb = ((15.0) / (180.0) * (PI_));
    if (prm->mobility_model == SCORE_MOBILITY_ROLLETT_HOLM)
        return 1.0 - (prm->RH_cut * exp(-1.0 * prm->RH_trans * pow((theta / lagb), prm->RH_exponent)));
    if (theta <= lagb) return -1.0;
    double maxDev40_111 = ((10.0) / (180.0) * (PI_));
    double _sqrt3 = 1 / sqrt(3.0);
    double oneNinth = 1.0 / 9.0;
    double qdis[4] = {1.0, 0.0, 0.0, 0.0};
    disori_quat(q1, q2, qdis);
    double m40_111[4] = {cos(oneNinth * PI_), _sqrt3 * sin(oneNinth * PI_), _sqrt3 * sin(oneNinth * PI_), _sqrt3 * sin(oneNinth * PI_)};
    double dev = disori_angle(qdis, m40_111);
    double w = 0.0;
    if (dev < maxDev40_111) w = cos(0.5 * PI_ * dev / maxDev40_111) * cos(0.5 * PI_ * dev / maxDev40_111);
    return w;
}

/* ------------------------------------------------------------------ master-thread physics */
typedef struct {
    const score_params* p;
    double t, dt, T, G, b, Gbhalfsq, mLAGB, mHAGB, mGS, mRH, fr, pzmin, Pmax, rhomax, tend;
} phys;

static void ph_temperature(phys* s) {  /* caHdl::update_temperature, SCORE_Kernel.cpp:5318-5336 */
    const score_params* p = s->p;
    uint32_t i = 0;
    while (i < p->n_schedule && p->sched_time[i] < s->t) i++;
    if (i == 0) { s->T = p->sched_temp[0]; return; }
    if (i >= p->n_schedule) { s->T = p->sched_temp[p->n_schedule - 1]; return; }
    s->T = p->sched_temp[i - 1] + ((p->sched_temp[i] - p->sched_temp[i - 1]) / (p->sched_time[i] - p->sched_time[i - 1])) * (s->t - p->sched_time[i - 1]);
}
static void ph_atomistic(phys* s) {  /* update_atomisticproperties + get_shearmodulus, SCORE_GeneralPhysics.cpp:65-78 */
    double T = s->T;
    s->G = s->p->G0 * (-1.38e-9 * (T * T * T) + 1.21e-6 * (T * T) - 4.58e-4 * T + 1.00);
    s->b = s->p->bZeroCelsius;
    s->Gbhalfsq = 0.5 * s->G * (s->b * s->b);
}
static void ph_micro(phys* s) {  /* update_microchemistry, SCORE_Kernel.cpp:5370-5406 */
    const score_params* p = s->p;
    if (p->zener_model == SCORE_ZENER_NONE) { s->fr = 0.0; s->pzmin = 0.0; return; }
    if (p->zener_model == SCORE_ZENER_CONSTANT) { s->fr = p->zener_fr[0]; s->pzmin = p->zener_alpha * p->zener_gamma * s->fr; return; }
    uint32_t i = 0;
    while (i < p->n_zener && p->zener_time[i] < s->t) i++;
    if (i == 0) s->fr = 0.0;
    if (i > 0 && i < p->n_zener) {
        double dfrdt = ((p->zener_fr[i] - p->zener_fr[i - 1]) / (p->zener_time[i] - p->zener_time[i - 1]));
        s->fr = p->zener_fr[i - 1] + dfrdt * (s->t - p->zener_time[i - 1]);
    }
    s->pzmin = p->zener_alpha * p->zener_gamma * s->fr;
}
static void ph_mobilities(phys* s) {  /* update_intrinsicmobilities, SCORE_Kernel.cpp:5354-5367 */
    const score_params* p = s->p;
    s->mLAGB = p->LAGBm0 * exp(-1.0 * p->LAGBHact / (KB * s->T));
    s->mHAGB = p->HAGBm0 * exp(-1.0 * p->HAGBHact / (KB * s->T));
    s->mGS = p->GSm0 * exp(-1.0 * p->GSHact / (KB * s->T));
    s->mRH = p->RH_HAGBm0 * exp(-1.0 * p->RH_HAGBHact / (KB * s->T));
}
static double ph_zener(const phys* s) {  /* get_zener, SCORE_Kernel.cpp:5448-5456 */
    if (s->p->zener_model == SCORE_ZENER_NONE) return 0.0;
    return (1.0 * s->p->zener_alpha * s->p->zener_gamma * s->fr);
}
static double ph_mobility(const phys* s, double P) {  /* get_currentintrinsicmobility, :5459-5470 */
    if (s->p->mobility_model == SCORE_MOBILITY_ROLLETT_HOLM) return (P * s->mRH);
    if (P < 0.0) return s->mLAGB;
    return ((P * s->mGS) + ((1.0 - P) * s->mHAGB));
}
static double ph_dtmin(const phys* s) {  /* get_dtmax_minimum and its parts, SCORE_Kernel.cpp:5519-5723 */
    const score_params* p = s->p;
    double mn = INFINITE_, d;
    /* temperature */
    {
        uint32_t i = 0;
        d = 1e-6;
        while (i < p->n_schedule && p->sched_time[i] < s->t) i++;
        if (i > 0) {
            if (i < p->n_schedule) {
                double dTdt = (fabs(p->sched_temp[i] - p->sched_temp[i - 1]) / (p->sched_time[i] - p->sched_time[i - 1]));
                if (dTdt <= 0.000277777777777777) dTdt = 0.000277777777777777;
                d = (1.0 / dTdt);
                double iv = p->sched_time[i] - p->sched_time[i - 1];
                if (d >= iv) d = iv;
            } else d = INFINITE_;
        }
        if (d < mn) mn = d;
    }
    /* recovery */
    d = INFINITE_;
    if (p->recovery_model == SCORE_RECOVERY_NES_VACCOREDIFF) {
        double Bx = PI_ * p->NesC3 * p->NesC5 * p->VacancyDiffD0 * exp(-1.0 * p->VacancyDiffHact / (KB * s->T));
        Bx = Bx / (p->NesKappa2 * (1.0 / pow(s->rhomax, 0.5)));
        double ex = (s->b * s->b) / (KB * s->T);
        double dr = Bx * exp(p->NesAlpha3 * p->NesKappa2 * s->G * s->b * ex);
        if (dr < (1.0 / pow(2.77e10, 0.5))) dr = (1.0 / pow(2.77e10, 0.5));
        d = (1.0 / pow(1.0e11, 0.5)) / dr;
    } else if (p->recovery_model == SCORE_RECOVERY_NES_SOLUTEDRAG) {
        double Bsa = p->NesC3 * s->b * p->SoluteDiffD0 * exp(-1.0 * p->SoluteDiffHact / (KB * s->T));
        double ex = (s->b * s->b) / (KB * s->T);
        double ls = p->SoluteLsPropFactor * pow(p->SoluteConcentration, (-2.0 / 3.0));
        double dr = Bsa * exp(p->NesAlpha3 * ls * s->G * s->b * ex / (1.0 / (s->rhomax * s->rhomax)));
        if (dr < (1.0 / pow(2.77e10, 0.5))) dr = (1.0 / pow(2.77e10, 0.5));
        d = (1.0 / pow(1.0e11, 0.5)) / dr;
    }
    if (d < mn) mn = d;
    /* zener */
    d = INFINITE_;
    if (p->zener_model == SCORE_ZENER_TIMEDEP) {
        uint32_t i = 0;
        d = 1e-6;
        while (i < p->n_zener && p->zener_time[i] < s->t) i++;
        if (i > 0) {
            if (i < p->n_zener) {
                double dp = p->zener_alpha * p->zener_gamma * (fabs(p->zener_fr[i] - p->zener_fr[i - 1]) / (p->zener_time[i] - p->zener_time[i - 1]));
                if (fabs(dp) <= 0.027777777) dp = 0.027777777;
                d = (100.0 / dp);
            } else d = INFINITE_;
        }
    }
    if (d < mn) mn = d;
    /* migration */
    if (p->mobility_model == SCORE_MOBILITY_ROLLETT_HOLM) {
        double mm = p->RH_HAGBm0 * exp(-1.0 * p->RH_HAGBHact / (KB * s->T));
        double vm = mm * ((s->Gbhalfsq * s->rhomax) - s->pzmin);
        d = ((p->maxfillperstep * p->cellsize) / vm);
    } else {
        double mgs = p->GSm0 * exp(-1.0 * p->GSHact / (KB * s->T));
        double mhagb = p->HAGBm0 * exp(-1.0 * p->HAGBHact / (KB * s->T));
        double m_max = (s->Pmax * mgs) + ((1.0 - s->Pmax) * mhagb);
        if (s->Pmax < (0.0 - 1e-6)) m_max = p->LAGBm0 * exp(-1.0 * p->LAGBHact / (KB * s->T));
        double v_max = m_max * ((s->Gbhalfsq * s->rhomax) - s->pzmin);
        d = ((p->maxfillperstep * p->cellsize) / v_max);
    }
    if (d < mn) mn = d;
    return mn;
}
/* update_deformedsubstructure, SCORE_Kernel.cpp:5409-5437, SCORE_RecoveryModels.cpp:50-126;
 * the hyperbolic law rho0/(1+kt) is not in the reference */
static void ph_recovery(const phys* s, double* rho, const double* rho0, uint32_t n) {
    const score_params* p = s->p;
    if (p->recovery_model == SCORE_RECOVERY_NES_VACCOREDIFF) {
        double B = PI_ * p->NesC3 * p->NesC5 * p->VacancyDiffD0 * exp(-1.0 * p->VacancyDiffHact / (KB * s->T));
        B /= p->NesKappa2;
        double ex = (s->b * s->b) / (KB * s->T);
        double et = exp(p->NesAlpha3 * p->NesKappa2 * s->G * s->b * ex);
        for (uint32_t g = 0; g < n; g++) {
            double r_t = 1.0 / pow(rho[g], 0.5);
            double Bx = (B / r_t) * et;
            double r_tdt = (Bx * s->dt) + r_t;
            rho[g] = 1.0 / (r_tdt * r_tdt);
        }
    } else if (p->recovery_model == SCORE_RECOVERY_MICHALAKPAXTON) {
        double tm = s->t / 60.0;
        double f = 0.25 * pow((1 + (tm / 0.3605)), -1.0) + 0.75 * pow((1 + (tm / 5.2824)), -0.5);
        for (uint32_t g = 0; g < n; g++) rho[g] = rho0[g] * (f * f);
    } else if (p->recovery_model == SCORE_RECOVERY_HYPERBOLIC) {
        double f = 1.0 + p->recovery_k * s->t;
        for (uint32_t g = 0; g < n; g++) rho[g] = rho0[g] / f;
    }
}
/* update_myrhomax, SCORE_RecoveryModels.cpp:150-170 */
static double rhomax_of(const double* rho, const uint32_t* cnt, uint32_t n) {
    double best = -1.0;
    for (uint32_t g = 0; g < n; g++)
        if (cnt[g] > 0 && rho[g] > best) best = rho[g];
    return best >= RHOMAX_WELLANNEALED ? best : RHOMAX_WELLANNEALED;
}

/* ------------------------------------------------------------------ front lists */
typedef struct {
    uint8_t* act;  uint8_t* inf;  int32_t* x; int32_t* y; int32_t* z;
    double* fill;  double* P;  uint32_t* defg;  uint32_t* rxg;
    uint32_t cap, never;       /* ntotalRXFront, nextSlotNeverActiveRXFront */
    uint32_t* rec; uint32_t reccap, rec_first, rec_next;  /* recycling list */
    uint32_t* full; uint32_t nfull, fullcap;
    int growable;
} flist;

static int fl_grow(flist* f, uint32_t need) {
    if (need <= f->cap) return 1;
    uint32_t nc = f->cap ? f->cap : 1024;
    while (nc < need) nc *= 2;
    f->act = realloc(f->act, nc); f->inf = realloc(f->inf, nc);
    f->x = realloc(f->x, nc * 4ull); f->y = realloc(f->y, nc * 4ull); f->z = realloc(f->z, nc * 4ull);
    f->fill = realloc(f->fill, nc * 8ull); f->P = realloc(f->P, nc * 8ull);
    f->defg = realloc(f->defg, nc * 4ull); f->rxg = realloc(f->rxg, nc * 4ull);
    if (!f->act || !f->inf || !f->x || !f->y || !f->z || !f->fill || !f->P || !f->defg || !f->rxg) return 0;
    for (uint32_t i = f->cap; i < nc; i++) {
        f->act[i] = 0; f->inf[i] = 26; f->x[i] = f->y[i] = f->z[i] = -1; f->fill[i] = 0.0; f->P[i] = -1.0;
        f->defg[i] = f->rxg[i] = 4096000001u;
    }
    f->cap = nc;
    return 1;
}
static void fl_free(flist* f) {
    free(f->act); free(f->inf); free(f->x); free(f->y); free(f->z); free(f->fill); free(f->P);
    free(f->defg); free(f->rxg); free(f->rec); free(f->full);
}

typedef struct {
    const score_params* p;
    phys ph;
    uint32_t nx, ny, nz, nxy, ndefg, nrxg;
    uint64_t N;
    uint32_t* grid;
    flist f[2];                 /* 0 Inside, 1 Border */
    uint32_t border_ref_cap;
    const double *rq, *dq;
    const double* ptab;
    double* pcache;
    uint32_t *rxg_cnt, *defg_cnt;
    double *rho, *rho0;
    double regPmax;             /* reg_myMobilityWeightMax */
    int status;
    uint64_t nnew;
} sim;

static double weight(sim* s, uint32_t r, uint32_t g) {
    uint64_t i = (uint64_t)r * s->ndefg + g;
    if (s->ptab) return s->ptab[i];
    if (s->pcache) {
        double v = s->pcache[i];
        if (v == v) return v;
        v = oracle_mobility_weight(s->p, s->rq + 4 * (size_t)r, s->dq + 4 * (size_t)g);
        s->pcache[i] = v;
        return v;
    }
    return oracle_mobility_weight(s->p, s->rq + 4 * (size_t)r, s->dq + 4 * (size_t)g);
}

/* omp_getNextFreeSlotInRXFront{Inside,Border}, SCORE_Kernel.cpp:3757-3874 */
static uint32_t next_slot(sim* s, int L, int recycle) {
    flist* f = &s->f[L];
    if (recycle && f->rec_next < f->rec_first) return f->rec[f->rec_next++];
    if (L == 1 && !f->growable && f->never >= s->border_ref_cap) { s->status = SCORE_ERR_BORDER_CAPACITY; return 0xFFFFFFFFu; }
    if (f->never >= f->cap && !fl_grow(f, f->never + 1)) { s->status = SCORE_ERR_NOMEM; return 0xFFFFFFFFu; }
    return f->never++;
}

/* ompshar_sim_myCA_calcGrowthStep{Inside,Border}, SCORE_Kernel.cpp:4046-4249 */
static const double SF[27] = {0.6494, 0.7957, 0.6494, 0.7957, 1.0000, 0.7957, 0.6494, 0.7957, 0.6494, 0.7957, 1.0000, 0.7957, 1.0000,
                              1.0000, 0.7957, 1.0000, 0.7957, 0.6494, 0.7957, 0.6494, 0.7957, 1.0000, 0.7957, 0.6494, 0.7957, 0.6494, 1.0};
static void grow(sim* s, int L, uint64_t* Sv, double* dV) {
    flist* f = &s->f[L];
    f->nfull = 0; f->rec_next = 0; f->rec_first = 0;
    uint64_t act = 0;
    double dv = 0.0;
    const double cinv = 1.0 / s->p->cellsize;
    const double zen = ph_zener(&s->ph);
    for (uint32_t c = 0; c < f->never; c++) {
        if (f->act[c]) {
            act++;
            double m = ph_mobility(&s->ph, f->P[c]);
            double p = (s->ph.Gbhalfsq * (s->rho[f->defg[c]] - RHO_RX)) - zen;
            if (p > 5.0e-16) {
                double v = m * p;
                v *= SF[f->inf[c]];
                f->fill[c] = f->fill[c] + (v * s->ph.dt * cinv);
                dv = dv + (v * s->ph.dt * cinv);
                if (f->fill[c] >= 1.0) {
                    if (f->nfull >= f->fullcap) { f->fullcap = f->fullcap ? 2 * f->fullcap : 1024; f->full = realloc(f->full, 4ull * f->fullcap); }
                    f->full[f->nfull++] = c;
                }
            }
            continue;
        }
        if (f->rec_first < f->reccap) f->rec[f->rec_first++] = c;  /* append_to_recycling_*_list */
    }
    *Sv += act;
    *dV += dv;
}

/* omp_infect_OutOfRXFront{Inside,Border}, SCORE_Kernel.cpp:4252-4556 (one region) */
static void infect(sim* s, int L, uint32_t src, int dest_border_from_inside, int dx, int dy, int dz, uint8_t code, double carry) {
    flist* f = &s->f[L];
    int x = f->x[src] + dx, y = f->y[src] + dy, z = f->z[src] + dz;
    int dest;
    if (L == 0) {
        dest = dest_border_from_inside;
    } else {
        if (x < 0) x += (int)s->nx;
        if (x >= (int)s->nx) x -= (int)s->nx;
        if (y < 0) y += (int)s->ny;
        if (y >= (int)s->ny) y -= (int)s->ny;
        if (s->p->boundary == SCORE_BOUNDARY_REFERENCE) {
            if (z < 0 || z >= (int)s->nz) return;
        } else {
            if (z < 0) z += (int)s->nz;
            if (z >= (int)s->nz) z -= (int)s->nz;
        }
        int inside = x > 0 && x < (int)s->nx - 1 && y > 0 && y < (int)s->ny - 1 && z > 0 && z < (int)s->nz - 1;
        dest = inside ? 0 : 1;
    }
    uint32_t t = (uint32_t)x + s->nx * ((uint32_t)y + s->ny * (uint32_t)z);
    uint32_t g = s->grid[t];
    if (g >= s->ndefg || g == CURRENTLY_INFECTED) return;
    s->grid[t] = CURRENTLY_INFECTED;
    uint32_t slot = next_slot(s, dest, 1);
    if (slot == 0xFFFFFFFFu) return;
    flist* d = &s->f[dest];
    d->act[slot] = 1; d->inf[slot] = code; d->x[slot] = x; d->y[slot] = y; d->z[slot] = z; d->fill[slot] = carry;
    d->P[slot] = f->P[src];
    if (f->defg[src] != g) d->P[slot] = weight(s, f->rxg[src], g);
    if (d->P[slot] >= s->regPmax) s->regPmax = d->P[slot];
    d->rxg[slot] = f->rxg[src];
    d->defg[slot] = g;
    s->nnew++;
}

/* ompshar_sim_myCA_updateFullRX{Inside,Border}, SCORE_Kernel.cpp:4559-4774 */
static const int8_t DX[26] = {-1, 0, 1, -1, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1};
static const int8_t DY[26] = {-1, -1, -1, 0, 0, 1, 1, 1, 1, 1, 1, -1, -1, -1, 0, 0, 0, -1, -1, -1, 0, 0, 0, 1, 1, 1};
static const int8_t DZ[26] = {0, 0, 0, 0, 0, 0, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
static const uint8_t CODE[26] = {16, 15, 14, 13, 12, 11, 10, 9, 19, 18, 17, 25, 24, 23, 22, 21, 20, 8, 7, 6, 5, 4, 3, 2, 1, 0};
static const uint8_t CLS[26] = {2, 1, 2, 1, 1, 2, 1, 2, 3, 2, 3, 3, 2, 3, 2, 1, 2, 3, 2, 3, 2, 1, 2, 3, 2, 3};

static uint64_t update_full(sim* s, int L) {
    flist* f = &s->f[L];
    for (uint32_t k = 0; k < f->nfull; k++) {
        uint32_t c = f->full[k];
        double overshoot = f->fill[c] - 1.0;
        double carry[4] = {0.0, overshoot * 0.0682, overshoot * 0.0542, overshoot * 0.0484};
        int into_border = 1;
        if (L == 0 && f->x[c] > 1 && f->x[c] < (int)s->nx - 2 && f->y[c] > 1 && f->y[c] < (int)s->ny - 2 && f->z[c] > 1 && f->z[c] < (int)s->nz - 2)
            into_border = 0;
        for (int d = 0; d < 26; d++) {
            infect(s, L, c, into_border, DX[d], DY[d], DZ[d], CODE[d], carry[CLS[d]]);
            if (s->status != SCORE_OK) return 0;
        }
        uint32_t cell = (uint32_t)f->x[c] + s->nx * ((uint32_t)f->y[c] + s->ny * (uint32_t)f->z[c]);
        s->grid[cell] = s->ndefg + f->rxg[c];
        s->rxg_cnt[f->rxg[c]] += 1;
        s->defg_cnt[f->defg[c]] -= 1;
        f->act[c] = 0;
        f->fill[c] = 0.0;
    }
    return f->nfull;
}

/* ompshar_defragmentation, SCORE_Kernel.cpp:3877-3937 */
static void defragment(flist* f) {
    uint32_t first = 0;
    while (first < f->cap && f->act[first]) first++;
    uint32_t cont = first;
    for (uint32_t c = first + 1; c < f->never; c++) {
        if (f->act[c]) {
            f->act[cont] = f->act[c]; f->inf[cont] = f->inf[c]; f->x[cont] = f->x[c]; f->y[cont] = f->y[c]; f->z[cont] = f->z[c];
            f->fill[cont] = f->fill[c]; f->P[cont] = f->P[c]; f->defg[cont] = f->defg[c]; f->rxg[cont] = f->rxg[c];
            cont++;
        }
    }
    f->never = cont;
}

/* ompshar_sim_myCA_sitesaturatedNucleation + infect_JuvenileNucleation, SCORE_GrowthMachine.cpp:50-189 */
static uint32_t place_nuclei(sim* s, const uint32_t* site, const double* tincub, uint8_t* considered, double tnow) {
    uint32_t n = 0;
    for (uint32_t r = 0; r < s->nrxg; r++) {
        if (considered[r] || (tincub && tincub[r] > tnow)) continue;
        considered[r] = 1;
        uint32_t w = site[r];
        uint32_t z = w / s->nxy, rem = w - s->nxy * z, y = rem / s->nx, x = rem - s->nx * y;
        uint32_t g = s->grid[w];
        if (g >= s->ndefg || g == CURRENTLY_INFECTED) continue;
        s->grid[w] = CURRENTLY_INFECTED;
        double PP = weight(s, r, g);
        int inside = x > 0 && x < s->nx - 1 && y > 0 && y < s->ny - 1 && z > 0 && z < s->nz - 1;
        int L = inside ? 0 : 1;
        uint32_t slot = next_slot(s, L, 0);
        if (slot == 0xFFFFFFFFu) return n;
        flist* f = &s->f[L];
        f->act[slot] = 1; f->inf[slot] = 26; f->x[slot] = (int)x; f->y[slot] = (int)y; f->z[slot] = (int)z;
        f->fill[slot] = 1.0; f->defg[slot] = g; f->rxg[slot] = r; f->P[slot] = PP;
        if (PP >= s->regPmax) s->regPmax = PP;
        n++;
    }
    return n;
}

/* the step loop's state between oracle_advance calls */
struct oracle_sim {
    sim S;
    const uint32_t* site;
    const double* tincub;
    uint8_t* considered;
    double Xcells, X;
    uint32_t step, it, defrag_cnt, nnuc;
    double dt0, Pmax0;
    /* grain-evolution log: snapshots taken so far, next logpoint */
    uint32_t nlog, logcap, log_next;
    double *log_t, *log_X;
    uint32_t *log_step, *log_sv, *log_counts, *log_area;
};

/* labels by the clarify rule (ompcrit_clarify_status_infectedcells, SCORE_Io_Characterization.cpp:925-1000):
   the grid, with every ACTIVE front cell as its deformed grain below fill 0.5 and its rx grain above */
static void labels_now(const sim* s, uint32_t* labels) {
    memcpy(labels, s->grid, s->N * 4);
    for (int L = 0; L < 2; L++) {
        const flist* f = &s->f[L];
        for (uint32_t c = 0; c < f->never; c++) {
            if (!f->act[c]) continue;
            uint32_t cell = (uint32_t)f->x[c] + s->nx * ((uint32_t)f->y[c] + s->ny * (uint32_t)f->z[c]);
            labels[cell] = (f->fill[c] < 0.5) ? f->defg[c] : s->ndefg + f->rxg[c];
        }
    }
}

/* log_OUTPUT_Diehl's grain-evolution branch (SCORE_OnTheFlyCharacterization.cpp:646-650), taken after the
   master block's counts and before t += dt: log_grainevo (:478-531: t, X, step, 32-bit Sv, every grain's
   cell count, deformed then rx) and the RX area profile of log_rxareaprofile(threshold) (:274-384: per z
   slice the cells of the rx grains whose section has at least `threshold` cells, and the rest) */
static int log_snapshot(oracle_sim* o, uint64_t Sv) {
    sim* s = &o->S;
    const uint32_t G = s->ndefg + s->nrxg, nz = s->nz, nxy = s->nxy;
    if (o->nlog == o->logcap) {
        uint32_t nc = o->logcap ? 2 * o->logcap : 16;
        o->log_t = realloc(o->log_t, nc * 8ull); o->log_X = realloc(o->log_X, nc * 8ull);
        o->log_step = realloc(o->log_step, nc * 4ull); o->log_sv = realloc(o->log_sv, nc * 4ull);
        o->log_counts = realloc(o->log_counts, (uint64_t)nc * G * 4); o->log_area = realloc(o->log_area, (uint64_t)nc * 2 * nz * 4);
        if (!o->log_t || !o->log_X || !o->log_step || !o->log_sv || !o->log_counts || !o->log_area) return 0;
        o->logcap = nc;
    }
    const uint32_t k = o->nlog++;
    o->log_t[k] = s->ph.t; o->log_X[k] = o->X; o->log_step[k] = o->step; o->log_sv[k] = (uint32_t)Sv;
    uint32_t* cnt = o->log_counts + (uint64_t)k * G;
    memcpy(cnt, s->defg_cnt, s->ndefg * 4ull);
    memcpy(cnt + s->ndefg, s->rxg_cnt, s->nrxg * 4ull);
    uint32_t* lab = malloc(s->N * 4);
    uint32_t* sec = calloc(s->nrxg ? s->nrxg : 1, 4);
    if (!lab || !sec) { free(lab); free(sec); return 0; }
    labels_now(s, lab);
    uint32_t* area = o->log_area + (uint64_t)k * 2 * nz;
    const uint32_t thr = s->p->rxarea_threshold;
    for (uint32_t z = 0; z < nz; z++) {
        const uint32_t* sl = lab + (uint64_t)z * nxy;
        for (uint32_t i = 0; i < nxy; i++)
            if (sl[i] >= s->ndefg && sl[i] < s->ndefg + s->nrxg) sec[sl[i] - s->ndefg]++;
        uint32_t rx = 0;
        for (uint32_t r = 0; r < s->nrxg; r++) {
            if (sec[r] >= thr) rx += sec[r];
            sec[r] = 0;
        }
        area[2 * z] = rx;
        area[2 * z + 1] = nxy - rx;
    }
    free(lab); free(sec);
    return 1;
}

oracle_sim* oracle_create(const score_params* p, const uint32_t* grid, const double* defg_q, const double* defg_rho0, uint32_t ndefg,
                          const double* rxg_q, const uint32_t* rxg_site, const double* rxg_tincub, uint32_t nrxg,
                          const double* ptable) {
    oracle_sim* o = calloc(1, sizeof *o);
    if (!o) return NULL;
    sim* s = &o->S;
    s->p = p; s->nx = p->nx; s->ny = p->ny; s->nz = p->nz; s->nxy = p->nx * p->ny;
    s->N = (uint64_t)p->nx * p->ny * p->nz;
    s->ndefg = ndefg; s->nrxg = nrxg; s->rq = rxg_q; s->dq = defg_q; s->ptab = ptable;
    s->status = SCORE_OK;
    s->grid = malloc(s->N * 4);
    memcpy(s->grid, grid, s->N * 4);
    s->rxg_cnt = calloc(nrxg ? nrxg : 1, 4);
    s->defg_cnt = calloc(ndefg, 4);
    s->rho = malloc(ndefg * 8ull); s->rho0 = malloc(ndefg * 8ull);
    memcpy(s->rho0, defg_rho0, ndefg * 8ull); memcpy(s->rho, defg_rho0, ndefg * 8ull);
    if (!ptable && (uint64_t)nrxg * ndefg <= (1ull << 26)) {
        s->pcache = malloc((uint64_t)nrxg * ndefg * 8 + 8);
        for (uint64_t i = 0; i < (uint64_t)nrxg * ndefg; i++) s->pcache[i] = NAN;
    }
    for (uint64_t i = 0; i < s->N; i++) s->defg_cnt[s->grid[i]]++;  /* solve_REPLACE_CA_STRUCTURE counts */
    s->border_ref_cap = 2 * ((p->nx * p->ny) + (p->nx * p->nz) + (p->ny * p->nz));
    /* ompshar_init_myRXFront{Inside,Border}, SCORE_Kernel.cpp:3587-3710 */
    s->f[0].reccap = (uint32_t)(p->initial_cache * (double)s->N * p->maxfillperstep * 3.0);
    s->f[1].reccap = (uint32_t)((double)s->border_ref_cap * p->maxfillperstep * 3.0);
    s->f[1].growable = p->border_policy == SCORE_BORDER_GROW;
    for (int L = 0; L < 2; L++) {
        s->f[L].rec = malloc(4ull * (s->f[L].reccap + 1));
        fl_grow(&s->f[L], 1024);
    }
    o->site = rxg_site;
    o->tincub = rxg_tincub;
    o->considered = calloc(nrxg ? nrxg : 1, 1);

    /* solve_RXGROWTH prologue, SCORE_Kernel.cpp:6513-6530 */
    phys* ph = &s->ph;
    ph->p = p; ph->t = 0.0; ph->T = 25.0 + 273.15; ph->fr = 0.0; ph->pzmin = 0.0; ph->Pmax = 0.0;
    ph->tend = 0.0;
    for (uint32_t i = 0; i < p->n_schedule; i++) if (p->sched_time[i] >= ph->tend) ph->tend = p->sched_time[i];
    ph->rhomax = rhomax_of(s->rho, s->defg_cnt, ndefg);
    ph_temperature(ph); ph_atomistic(ph); ph_mobilities(ph);
    ph->dt = ph_dtmin(ph);
    o->dt0 = ph->dt;
    s->regPmax = 0.0;
    o->nnuc = place_nuclei(s, rxg_site, rxg_tincub, o->considered, 0.0);
    if (s->regPmax >= ph->Pmax) ph->Pmax = s->regPmax;
    o->Pmax0 = ph->Pmax;
    return o;
}

int oracle_advance(oracle_sim* o, double x_target, uint32_t max_steps, oracle_step* trace, uint32_t trace_cap, oracle_out* out) {
    sim* s = &o->S;
    const score_params* p = s->p;
    phys* ph = &s->ph;
    const double xt = x_target < 0 ? p->xmax : x_target;
    uint32_t done = 0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (; o->it < 1000000u && s->status == SCORE_OK; o->it++) {
        if ((o->Xcells >= (double)s->N) || (o->X > xt) || (o->it > p->nmax) || (ph->t > ph->tend) || (ph->t > p->tmax)) break;
        if (max_steps && done >= max_steps) break;
        uint32_t newnuc = o->tincub ? place_nuclei(s, o->site, o->tincub, o->considered, ph->t) : 0;
        o->nnuc += newnuc;
        if (p->defragmentation && o->defrag_cnt < p->n_defrag && o->Xcells >= p->defrag_x[o->defrag_cnt] * (double)s->N) {
            defragment(&s->f[0]);
            defragment(&s->f[1]);
            o->defrag_cnt++;
        }
        uint64_t Sv = 0;
        double dV = 0.0;
        s->nnew = 0;
        grow(s, 0, &Sv, &dV);
        grow(s, 1, &Sv, &dV);
        uint64_t nfull = update_full(s, 0);
        nfull += update_full(s, 1);
        if (s->status != SCORE_OK) break;
        /* master block, SCORE_Kernel.cpp:6691-6740 */
        double mymob = 0.0;
        if (s->regPmax >= mymob) mymob = s->regPmax;
        ph->Pmax = mymob;
        o->Xcells = o->Xcells + (double)nfull;
        o->X = (o->Xcells / (double)s->N);
        ph->rhomax = rhomax_of(s->rho, s->defg_cnt, s->ndefg);
        double rhomax_step = ph->rhomax, dt_used = ph->dt;
        if (o->log_next < p->n_logpoints && o->Xcells >= p->logpoint_x[o->log_next] * (double)s->N) {
            if (!log_snapshot(o, Sv)) { s->status = SCORE_ERR_NOMEM; break; }
            o->log_next++;
        }
        ph->t += ph->dt;
        ph_temperature(ph); ph_atomistic(ph); ph_micro(ph); ph_mobilities(ph);
        ph_recovery(ph, s->rho, s->rho0, s->ndefg);
        ph->dt = ph_dtmin(ph);
        o->step++;
        if (trace && done < trace_cap) {
            oracle_step* r = &trace[done];
            memset(r, 0, sizeof *r);
            r->step = o->step; r->n_nuclei = newnuc; r->t = ph->t; r->dt = ph->dt; r->dt_used = dt_used; r->Xcells = o->Xcells; r->X = o->X;
            r->Sv = Sv; r->n_full = nfull; r->n_new = s->nnew; r->Pmax = ph->Pmax; r->rhomax = rhomax_step; r->dXstep = dV;
            r->next_never[0] = s->f[0].never; r->next_never[1] = s->f[1].never;
            r->n_recycled[0] = s->f[0].rec_first; r->n_recycled[1] = s->f[1].rec_first;
        }
        done++;
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (out) {
        out->n_steps = done; out->status = s->status; out->dt0 = o->dt0; out->Pmax0 = o->Pmax0; out->n_nuclei = o->nnuc;
        out->seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    }
    return s->status;
}

int oracle_done(const oracle_sim* o, double x_target) {
    const sim* s = &o->S;
    const double xt = x_target < 0 ? s->p->xmax : x_target;
    return s->status != SCORE_OK || (o->Xcells >= (double)s->N) || (o->X > xt) || (o->it > s->p->nmax) || (s->ph.t > s->ph.tend) ||
           (s->ph.t > s->p->tmax) || o->it >= 1000000u;
}

double oracle_time(const oracle_sim* o) { return o->S.ph.t; }

uint32_t oracle_log_count(const oracle_sim* o) { return o->nlog; }

int oracle_log_get(const oracle_sim* o, uint32_t i, double* t, double* X, uint32_t* step, uint32_t* sv, uint32_t* counts,
                   uint32_t* area) {
    const sim* s = &o->S;
    if (i >= o->nlog) return SCORE_ERR_ARG;
    const uint32_t G = s->ndefg + s->nrxg;
    if (t) *t = o->log_t[i];
    if (X) *X = o->log_X[i];
    if (step) *step = o->log_step[i];
    if (sv) *sv = o->log_sv[i];
    if (counts) memcpy(counts, o->log_counts + (uint64_t)i * G, G * 4ull);
    if (area) memcpy(area, o->log_area + (uint64_t)i * 2 * s->nz, 2ull * s->nz * 4);
    return SCORE_OK;
}

void oracle_finish(const oracle_sim* o, uint32_t* labels, uint32_t* rxg_counts, uint32_t* defg_counts) {
    const sim* s = &o->S;
    /* final labels, ompcrit_clarify_status_infectedcells (SCORE_Io_Characterization.cpp:925-1000) */
    if (labels) labels_now(s, labels);
    if (rxg_counts) memcpy(rxg_counts, s->rxg_cnt, s->nrxg * 4ull);
    if (defg_counts) memcpy(defg_counts, s->defg_cnt, s->ndefg * 4ull);
}

void oracle_destroy(oracle_sim* o) {
    if (!o) return;
    sim* s = &o->S;
    fl_free(&s->f[0]); fl_free(&s->f[1]);
    free(s->grid); free(s->rxg_cnt); free(s->defg_cnt); free(s->rho); free(s->rho0); free(s->pcache); free(o->considered);
    free(o->log_t); free(o->log_X); free(o->log_step); free(o->log_sv); free(o->log_counts); free(o->log_area);
    free(o);
}

/* ------------------------------------------------------------------ ensemble post-processing */
/* caHdl::get_interpCellCount, SCORE_SolitaryUnitAveraging.cpp:1304-1365: the final count at or after the
   end of the run, else linear between the logged snapshots that frame `when` (the first snapshot
   before the first log time, the last one after the last); the scan stops at the end of the log */
double oracle_interp_count(const oracle_evo* e, uint32_t id, double when) {
    const uint32_t G = e->ndefg + e->nrxg;
    if (when >= e->tsimend || e->nsnap == 0) return (double)e->final_counts[id];  /* the reference indexes an empty log there */
    uint32_t i = 0;
    while (i < e->nsnap && e->t[i] < when) i++;
    if (i > 0 && i < e->nsnap) {
        double ti1 = e->t[i - 1];
        double cnti1 = e->counts[(uint64_t)(i - 1) * G + id];
        double ti = e->t[i];
        double cnti = e->counts[(uint64_t)i * G + id];
        return cnti1 + ((when - ti1) * ((cnti - cnti1) / (ti - ti1)));
    }
    if (i == 0) return (double)e->counts[id];
    return (double)e->counts[(uint64_t)(e->nsnap - 1) * G + id];
}

/* ensembleHdl::postprocess_init + postprocess_initrediscrtimes (SCORE_SolitaryUnitAveraging.cpp:50-80, 510-540):
   nslots equidistant times over [0, latest end time], each the end of its interval */
static double rediscr_times(const oracle_evo* doms, uint32_t ndom, uint32_t nslots, double* t_out) {
    double tmax = 0.0;
    for (uint32_t d = 0; d < ndom; d++) if (doms[d].tsimend >= tmax) tmax = doms[d].tsimend;
    const double ttmin = 0.0, dt = (tmax - ttmin) / ((double)(nslots - 1));
    for (uint32_t n = 0; n < nslots; n++) t_out[n] = ttmin + ((double)(n + 1) * dt);
    return tmax;
}

/* ensembleHdl::postprocess_rediscr_kinetics, SCORE_SolitaryUnitAveraging.cpp:546-670: per time slot the
   recrystallized volume of the ensemble, sum over domains of (box volume - interpolated deformed volume) */
void oracle_rediscr_kinetics(const oracle_evo* doms, uint32_t ndom, uint32_t nslots, double* t_out, double* vol_out,
                             double* boxvol_out) {
    rediscr_times(doms, ndom, nslots, t_out);
    double* dv = malloc(nslots * 8ull);
    double box = 0.0;
    for (uint32_t n = 0; n < nslots; n++) vol_out[n] = 0.0;
    for (uint32_t d = 0; d < ndom; d++) {
        box = box + doms[d].nboxvol;
        for (uint32_t n = 0; n < nslots; n++) dv[n] = 0.0;
        for (uint32_t g = 0; g < doms[d].ndefg; g++)
            for (uint32_t n = 0; n < nslots; n++) dv[n] = dv[n] + oracle_interp_count(&doms[d], g, t_out[n]);
        for (uint32_t n = 0; n < nslots; n++) vol_out[n] = vol_out[n] + (doms[d].nboxvol - dv[n]);
    }
    if (boxvol_out) *boxvol_out = box;
    free(dv);
}

/* ensembleHdl::postprocess_rediscr_macrotexture, SCORE_SolitaryUnitAveraging.cpp:673-804: per time slot and
   orientation class the interpolated volume of the ensemble's grains, deformed then rx, [slot][class] */
void oracle_rediscr_macrotexture(const oracle_evo* doms, uint32_t ndom, uint32_t nslots, uint32_t nclass, double* t_out,
                                 double* vol_out) {
    rediscr_times(doms, ndom, nslots, t_out);
    const uint64_t M = (uint64_t)nslots * nclass;
    double* dv = malloc(M * 8);
    for (uint64_t k = 0; k < M; k++) vol_out[k] = 0.0;
    for (uint32_t d = 0; d < ndom; d++) {
        const oracle_evo* e = &doms[d];
        for (uint64_t k = 0; k < M; k++) dv[k] = 0.0;
        for (uint32_t g = 0; g < e->ndefg + e->nrxg; g++) {
            const uint32_t c = e->grain_class[g];
            for (uint32_t n = 0; n < nslots; n++) dv[(uint64_t)nclass * n + c] += oracle_interp_count(e, g, t_out[n]);
        }
        for (uint64_t k = 0; k < M; k++) vol_out[k] += dv[k];
    }
    free(dv);
}

int oracle_run(const score_params* p, const uint32_t* grid, const double* defg_q, const double* defg_rho0, uint32_t ndefg,
               const double* rxg_q, const uint32_t* rxg_site, const double* rxg_tincub, uint32_t nrxg, const double* ptable,
               double x_target, uint32_t max_steps, oracle_step* trace, uint32_t trace_cap, uint32_t* labels,
               uint32_t* rxg_counts, uint32_t* defg_counts, oracle_out* out) {
    oracle_sim* o = oracle_create(p, grid, defg_q, defg_rho0, ndefg, rxg_q, rxg_site, rxg_tincub, nrxg, ptable);
    if (!o) return SCORE_ERR_NOMEM;
    const int status = oracle_advance(o, x_target, max_steps, trace, trace_cap, out);
    oracle_finish(o, labels, rxg_counts, defg_counts);
    oracle_destroy(o);
    return status;
}

/* ------------------------------------------------------------------ percolation */
/* caHdl::binarize_partiallyrxed_microstructure, SCORE_OnTheFlyCharacterization.cpp:732-774: recrystallized
   and currently infected cells (grid value >= ndefg) are 1 */
void oracle_binarize(const oracle_sim* o, uint8_t* bin) {
    const sim* s = &o->S;
    for (uint64_t i = 0; i < s->N; i++) bin[i] = s->grid[i] >= s->ndefg ? 1 : 0;
}

static uint32_t uf_root(uint32_t* id, uint32_t p) {  /* UF::find_root with path compression, SCORE_PercAnalyzer.h:133-143 */
    uint32_t root = p;
    while (root != id[root]) root = id[root];
    while (p != root) { uint32_t q = id[p]; id[p] = root; p = q; }
    return root;
}
static uint32_t uf_merge(uint32_t* id, uint32_t* sz, uint32_t x, uint32_t y) {  /* UF::merge, :146-160 */
    uint32_t i = uf_root(id, x), j = uf_root(id, y);
    if (i == j) return i;
    if (sz[i] < sz[j]) { id[i] = j; sz[j] += sz[i]; return j; }
    id[j] = i; sz[i] += sz[j];
    return i;
}
static int cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return (x > y) - (x < y);
}

/* Clusters of the 1-cells, 6-connected, not periodic, in the reference's terms (percAnalyzer,
   SCORE_PercAnalyzer.cpp): labels 1..n in the order of each cluster's first cell (compactify, :334-390),
   0 outside every cluster; percolates when a cluster touches both faces of one axis (percolates,
   :500-615); sizes ascending (determine_clustersize_distr, :617-656).
   reference_scan = 1 runs the reference's sequential Hoshen-Kopelman scan itself (hk3d_core_nonperiodic,
   :161-226, with its union-find): labels are cell indices and 0 means "not recrystallized", so the
   origin cell never joins a cluster, and a cell whose three lower neighbours are all labelled merges only
   the lower two (:218-225), which can leave one true cluster split in two.
   reference_scan = 0 computes the true 6-connected clusters, the origin cell left out as the reference
   leaves it out. */
int oracle_percolation(const uint8_t* bin, uint32_t nx, uint32_t ny, uint32_t nz, int reference_scan, uint32_t* labels,
                       uint32_t* n_clusters, uint32_t* largest, int* percolates, uint32_t* spans, uint32_t* sizes) {
    const uint64_t N = (uint64_t)nx * ny * nz, nxy = (uint64_t)nx * ny;
    uint32_t* id = malloc(N * 4);
    uint32_t* uf = malloc(N * 4);
    uint32_t* sz = malloc(N * 4);
    if (!id || !uf || !sz) { free(id); free(uf); free(sz); return SCORE_ERR_NOMEM; }
    for (uint64_t i = 0; i < N; i++) { id[i] = bin[i] ? 1u : 0u; uf[i] = (uint32_t)i; sz[i] = 1; }
    for (uint32_t z = 0; z < nz; z++)
        for (uint32_t y = 0; y < ny; y++)
            for (uint32_t x = 0; x < nx; x++) {
                const uint64_t c = x + nx * ((uint64_t)y + (uint64_t)ny * z);
                if (id[c] != 1) continue;  /* only the cells still marked 1 (unlabelled) */
                uint32_t front = z == 0 ? 0 : id[c - nxy], bottom = y == 0 ? 0 : id[c - nx], left = x == 0 ? 0 : id[c - 1];
                if (reference_scan) {
                    int bl = left > 0, bb = bottom > 0, bf = front > 0;
                    if (!bl && !bb && !bf) id[c] = (uint32_t)c;
                    else if (bl && !bb && !bf) id[c] = left;
                    else if (!bl && bb && !bf) id[c] = bottom;
                    else if (!bl && !bb && bf) id[c] = front;
                    else if (bl && bb && !bf) id[c] = uf_merge(uf, sz, left, bottom);
                    else if (bl && !bb && bf) id[c] = uf_merge(uf, sz, left, front);
                    else if (!bl && bb && bf) id[c] = uf_merge(uf, sz, bottom, front);
                    else id[c] = uf_merge(uf, sz, bottom, front);
                } else {
                    if (c == 0) { id[c] = 0; continue; }
                    uint32_t lab = (uint32_t)c;
                    if (left) lab = uf_merge(uf, sz, lab, left);
                    if (bottom) lab = uf_merge(uf, sz, lab, bottom);
                    if (front) lab = uf_merge(uf, sz, lab, front);
                    id[c] = lab;
                }
            }
    /* compactify: new labels in the order of first appearance of each root */
    uint32_t* newkey = uf;  /* reuse as root -> new label map after resolving every root */
    uint32_t* root = sz;
    for (uint64_t i = 0; i < N; i++) root[i] = id[i] > 0 ? uf_root(uf, id[i]) : 0xFFFFFFFFu;
    for (uint64_t i = 0; i < N; i++) newkey[i] = 0;
    uint32_t n = 0;
    for (uint64_t i = 0; i < N; i++) {
        if (root[i] == 0xFFFFFFFFu) { labels[i] = 0; continue; }
        if (newkey[root[i]] == 0) newkey[root[i]] = ++n;
        labels[i] = newkey[root[i]];
    }
    free(id); free(uf); free(sz);
    /* sizes, faces */
    uint32_t* cnt = calloc(n + 1, 4);
    uint8_t* face = calloc(n + 1, 1);
    if (!cnt || !face) { free(cnt); free(face); return SCORE_ERR_NOMEM; }
    for (uint32_t z = 0; z < nz; z++)
        for (uint32_t y = 0; y < ny; y++)
            for (uint32_t x = 0; x < nx; x++) {
                const uint32_t l = labels[x + nx * ((uint64_t)y + (uint64_t)ny * z)];
                if (!l) continue;
                cnt[l]++;
                face[l] |= (x == 0 ? 1 : 0) | (x == nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == ny - 1 ? 8 : 0) |
                           (z == 0 ? 16 : 0) | (z == nz - 1 ? 32 : 0);
            }
    uint32_t big = 0, sp = 0;
    for (uint32_t l = 1; l <= n; l++) {
        if (cnt[l] > big) big = cnt[l];
        if ((face[l] & 3) == 3) sp |= 1;
        if ((face[l] & 12) == 12) sp |= 2;
        if ((face[l] & 48) == 48) sp |= 4;
    }
    if (sizes) { memcpy(sizes, cnt + 1, n * 4ull); qsort(sizes, n, 4, cmp_u32); }
    *n_clusters = n; *largest = big; *percolates = sp != 0; *spans = sp;
    free(cnt); free(face);
    return SCORE_OK;
}

