// Host FP64 model: .uds reader, master-thread physics and the mobility weight.
// Compiled with -ffp-contract=off; every expression keeps the reference's
// evaluation order (cited per function) so the doubles are bit-identical.
#include "host_model.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

namespace score {

// ---------------------------------------------------------------- mobility weight

// Hamilton product r = a (x) b in the ijk convention with P_EIJK = +1
// (mathMethods::multiply_quat_degraef, SCORE_Math.cpp:230-239).
static inline void quat_mul(const double a[4], const double b[4], double r[4]) {
    r[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    r[1] = b[0] * a[1] + a[0] * b[1] + (a[2] * b[3] - a[3] * b[2]);
    r[2] = b[0] * a[2] + a[0] * b[2] + (-(a[1] * b[3]) + a[3] * b[1]);
    r[3] = b[0] * a[3] + a[0] * b[3] + (a[1] * b[2] - a[2] * b[1]);
}

// The 24 candidate scalar parts of the cubic-symmetry-equivalent misorientations,
// arranged as six quaternions (Grimmer 1974; SCORE_Math.cpp:581-594).
static inline void grimmer_candidates(const double p[4], const double q[4], double c[6][4]) {
    const double qinv[4] = {q[0], -q[1], -q[2], -q[3]};
    double r[4];
    quat_mul(qinv, p, r);
    const double a = r[0], b = r[1], cc = r[2], d = r[3];
    const double fac = 1.0 / std::sqrt(2.0);
    c[0][0] = (a + b) * fac;  c[0][1] = (a - b) * fac;  c[0][2] = (cc + d) * fac; c[0][3] = (cc - d) * fac;
    c[1][0] = (a + cc) * fac; c[1][1] = (a - cc) * fac; c[1][2] = (b + d) * fac;  c[1][3] = (b - d) * fac;
    c[2][0] = (a + d) * fac;  c[2][1] = (a - d) * fac;  c[2][2] = (b + cc) * fac; c[2][3] = (b - cc) * fac;
    c[3][0] = (a + b + cc + d) * 0.5; c[3][1] = (a + b - cc - d) * 0.5; c[3][2] = (a - b + cc - d) * 0.5; c[3][3] = (a - b - cc + d) * 0.5;
    c[4][0] = (a + b + cc - d) * 0.5; c[4][1] = (a + b - cc + d) * 0.5; c[4][2] = (a - b + cc + d) * 0.5; c[4][3] = (a - b - cc - d) * 0.5;
    c[5][0] = a; c[5][1] = b; c[5][2] = cc; c[5][3] = d;
}

double disori_angle_cubic(const double p[4], const double q[4]) {
    double c[6][4];
    grimmer_candidates(p, q, c);
    double omega = 0.0;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 4; ++j)
            if (std::fabs(c[i][j]) > omega) omega = std::fabs(c[i][j]);
    if (omega < (1.0 - kDoubleAccuracy)) return 2.0 * std::acos(omega);
    return 0.0;
}

void disori_quat_cubic(const double p[4], const double q[4], double out[4]) {
    double c[6][4];
    grimmer_candidates(p, q, c);
    int mi = 0;
    double mx = 0.0;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 4; ++j)
            if (std::fabs(c[i][j]) > mx) { mx = std::fabs(c[i][j]); mi = i; }
    double s[4] = {std::fabs(c[mi][0]), std::fabs(c[mi][1]), std::fabs(c[mi][2]), std::fabs(c[mi][3])};
    std::sort(s, s + 4);  // ascending; the reference's bubble sort yields the same order of values
    out[0] = s[3]; out[1] = s[2]; out[2] = s[1]; out[3] = s[0];
}

double mobility_weight(const score_params& prm, const double qr[4], const double qd[4]) {
    const double lagb_hagb = (15.0) / (180.0) * (kPi);
    const double theta = disori_angle_cubic(qr, qd);
    if (prm.mobility_model == SCORE_MOBILITY_ROLLETT_HOLM) {
        return 1.0 - (prm.RH_cut * std::exp(-1.0 * prm.RH_trans * std::pow((theta / lagb_hagb), prm.RH_exponent)));
    }
    if (theta <= lagb_hagb) return -1.0;
    const double maxDev = (10.0) / (180.0) * (kPi);
    // The deviation from 40deg<111> is at least |theta - 40 deg| (triangle inequality of the
    // disorientation, a metric on orientations modulo the cubic group), so far from 40 deg the
    // weight is the reference's 0 without its second disorientation; the 1e-9 rad margin is
    // many orders above the rounding of either angle.
    if (std::fabs(theta - 2.0 * kPi / 9.0) > maxDev + 1e-9) return 0.0;
    const double sqrt3inv = 1 / std::sqrt(3.0);
    const double oneNinth = 1.0 / 9.0;
    double qdis[4];
    disori_quat_cubic(qr, qd, qdis);
    const double m40[4] = {std::cos(oneNinth * kPi), sqrt3inv * std::sin(oneNinth * kPi),
                           sqrt3inv * std::sin(oneNinth * kPi), sqrt3inv * std::sin(oneNinth * kPi)};
    const double dev = disori_angle_cubic(qdis, m40);
    double w = 0.0;
    if (dev < maxDev) {
        const double c = std::cos(0.5 * kPi * dev / maxDev);
        w = c * c;
    }
    return w;
}

void weight_constants(const score_params& prm, double* fac, double* lagb, double* maxdev, double m40[4], double* theta_sat) {
    *fac = 1.0 / std::sqrt(2.0);
    *lagb = (15.0) / (180.0) * (kPi);
    *maxdev = (10.0) / (180.0) * (kPi);
    const double sqrt3inv = 1 / std::sqrt(3.0);
    const double oneNinth = 1.0 / 9.0;
    m40[0] = std::cos(oneNinth * kPi);
    m40[1] = m40[2] = m40[3] = sqrt3inv * std::sin(oneNinth * kPi);
    // Rollett-Holm: once trans (theta/15deg)^expo exceeds 60, cut*exp(-60..) < 2^-60 for
    // cut < 1e7, so 1 - cut*exp(..) rounds to exactly 1.0 whatever libm's last bit
    *theta_sat = 1e300;
    if (prm.mobility_model == SCORE_MOBILITY_ROLLETT_HOLM && prm.RH_trans > 0.0 && prm.RH_exponent > 0.0 &&
        std::fabs(prm.RH_cut) < 1e7)
        *theta_sat = *lagb * std::pow(60.0 / prm.RH_trans, 1.0 / prm.RH_exponent) * (1.0 + 1e-6);
}

// ---------------------------------------------------------------- physics

void Physics::init(const score_params* p) {
    prm = p;
    t = 0.0; T = 25.0 + kToffset; fr = 0.0; pzmin = 0.0; Pmax = kDefaultPmax; rhomax = kRhomaxWellAnnealed;
    t_end = 0.0;  // caHdl::init_processing, SCORE_Kernel.cpp:5871-5884
    for (uint32_t i = 0; i < p->n_schedule; ++i)
        if (p->sched_time[i] >= t_end) t_end = p->sched_time[i];
}

// caHdl::update_temperature, SCORE_Kernel.cpp:5318-5336
void Physics::update_temperature() {
    const uint32_t n = prm->n_schedule;
    uint32_t i = 0;
    while (i < n && prm->sched_time[i] < t) i++;
    if (i == 0) { T = prm->sched_temp[0]; return; }
    if (i >= n) { T = prm->sched_temp[n - 1]; return; }
    T = prm->sched_temp[i - 1] + ((prm->sched_temp[i] - prm->sched_temp[i - 1]) / (prm->sched_time[i] - prm->sched_time[i - 1])) * (t - prm->sched_time[i - 1]);
}

// caHdl::update_atomisticproperties + get_shearmodulus (bcc iron), SCORE_Kernel.cpp:5339-5351,
// SCORE_GeneralPhysics.cpp:65-78
void Physics::update_atomistic() {
    G = prm->G0 * (-1.38e-9 * ((T) * (T) * (T)) + 1.21e-6 * ((T) * (T)) - 4.58e-4 * T + 1.00);
    b = prm->bZeroCelsius;
    Gbhalfsq = 0.5 * G * ((b) * (b));
}

// caHdl::update_microchemistry, SCORE_Kernel.cpp:5370-5406.  For a time-dependent drag at a
// time before the first table entry the reference reads index -1; here fr stays 0 instead.
void Physics::update_microchemistry() {
    if (prm->zener_model == SCORE_ZENER_NONE) { fr = 0.0; pzmin = 0.0; return; }
    if (prm->zener_model == SCORE_ZENER_CONSTANT) {
        fr = prm->zener_fr[0];
        pzmin = prm->zener_alpha * prm->zener_gamma * fr;
        return;
    }
    const uint32_t n = prm->n_zener;
    uint32_t i = 0;
    while (i < n && prm->zener_time[i] < t) i++;
    if (i == 0) fr = 0.0;
    if (i > 0 && i < n) {
        double dfrdt = ((prm->zener_fr[i] - prm->zener_fr[i - 1]) / (prm->zener_time[i] - prm->zener_time[i - 1]));
        fr = prm->zener_fr[i - 1] + dfrdt * (t - prm->zener_time[i - 1]);
    }
    pzmin = prm->zener_alpha * prm->zener_gamma * fr;
}

// caHdl::update_intrinsicmobilities, SCORE_Kernel.cpp:5354-5367
void Physics::update_mobilities() {
    mLAGB = prm->LAGBm0 * std::exp(-1.0 * prm->LAGBHact / (kBoltzmann * T));
    mHAGB = prm->HAGBm0 * std::exp(-1.0 * prm->HAGBHact / (kBoltzmann * T));
    mGS = prm->GSm0 * std::exp(-1.0 * prm->GSHact / (kBoltzmann * T));
    mRHHAGB = prm->RH_HAGBm0 * std::exp(-1.0 * prm->RH_HAGBHact / (kBoltzmann * T));
}

// caHdl::get_zener, SCORE_Kernel.cpp:5448-5456
double Physics::zener() const {
    if (prm->zener_model == SCORE_ZENER_NONE) return 0.0;
    return (1.0 * prm->zener_alpha * prm->zener_gamma * fr);
}

// caHdl::get_currentintrinsicmobility, SCORE_Kernel.cpp:5459-5470
double Physics::intrinsic_mobility(double P) const {
    if (prm->mobility_model == SCORE_MOBILITY_ROLLETT_HOLM) return (P * mRHHAGB);
    if (P < 0.0) return mLAGB;
    return ((P * mGS) + ((1.0 - P) * mHAGB));
}

// the grow step's driving force, SCORE_Kernel.cpp:4082
double Physics::driving_force(double rho) const {
    return (Gbhalfsq * (rho - kRhoRecrystallized)) - zener();
}

// caHdl::get_dtmax_instantslope_temp, SCORE_Kernel.cpp:5560-5591
double Physics::dt_temp() const {
    const uint32_t n = prm->n_schedule;
    uint32_t i = 0;
    double dtmax = kInitialDeltaT;
    while (i < n && prm->sched_time[i] < t) i++;
    if (i == 0) return dtmax;
    if (i < n) {
        double dTdt = (std::fabs(prm->sched_temp[i] - prm->sched_temp[i - 1]) / (prm->sched_time[i] - prm->sched_time[i - 1]));
        if (dTdt <= kSmallHeatRate) dTdt = kSmallHeatRate;
        dtmax = (kSmallHeat / dTdt);
        double dtintvl = prm->sched_time[i] - prm->sched_time[i - 1];
        if (dtmax >= dtintvl) dtmax = dtintvl;
        return dtmax;
    }
    return kInfinite;
}

// caHdl::get_dtmax_instantslope_rho, SCORE_Kernel.cpp:5594-5636
double Physics::dt_rho() const {
    const int m = prm->recovery_model;
    if (m == SCORE_RECOVERY_NES_VACCOREDIFF) {
        double Bx = kPi * prm->NesC3 * prm->NesC5 * prm->VacancyDiffD0 * std::exp(-1.0 * prm->VacancyDiffHact / (kBoltzmann * T));
        Bx = Bx / (prm->NesKappa2 * (1.0 / std::pow(rhomax, 0.5)));
        double exponent = ((b) * (b)) / (kBoltzmann * T);
        double drdtmax = Bx * std::exp(prm->NesAlpha3 * prm->NesKappa2 * G * b * exponent);
        if (drdtmax < (1.0 / std::pow(kSmallRecoveryRate, 0.5))) drdtmax = (1.0 / std::pow(kSmallRecoveryRate, 0.5));
        return (1.0 / std::pow(kSmallRho, 0.5)) / drdtmax;
    }
    if (m == SCORE_RECOVERY_NES_SOLUTEDRAG) {
        double Bsa = prm->NesC3 * b * prm->SoluteDiffD0 * std::exp(-1.0 * prm->SoluteDiffHact / (kBoltzmann * T));
        double exponent = ((b) * (b)) / (kBoltzmann * T);
        double ls = prm->SoluteLsPropFactor * std::pow(prm->SoluteConcentration, (-2.0 / 3.0));
        double drdtmax = Bsa * std::exp(prm->NesAlpha3 * ls * G * b * exponent / (1.0 / ((rhomax) * (rhomax))));
        if (drdtmax < (1.0 / std::pow(kSmallRecoveryRate, 0.5))) drdtmax = (1.0 / std::pow(kSmallRecoveryRate, 0.5));
        return (1.0 / std::pow(kSmallRho, 0.5)) / drdtmax;
    }
    return kInfinite;
}

// caHdl::get_dtmax_instantslope_zener, SCORE_Kernel.cpp:5639-5671
double Physics::dt_zener() const {
    if (prm->zener_model != SCORE_ZENER_TIMEDEP) return kInfinite;
    const uint32_t n = prm->n_zener;
    uint32_t i = 0;
    double dtmax = kInitialDeltaT;
    while (i < n && prm->zener_time[i] < t) i++;
    if (i == 0) return dtmax;
    if (i < n) {
        double dpzdt = prm->zener_alpha * prm->zener_gamma * (std::fabs(prm->zener_fr[i] - prm->zener_fr[i - 1]) / (prm->zener_time[i] - prm->zener_time[i - 1]));
        if (std::fabs(dpzdt) <= kSmallDraggingRate) dpzdt = kSmallDraggingRate;
        return (kSmallZenerForce / dpzdt);
    }
    return kInfinite;
}

// caHdl::get_dtmax_instantslope_cells, SCORE_Kernel.cpp:5519-5557
double Physics::dt_cells() const {
    if (prm->mobility_model == SCORE_MOBILITY_ROLLETT_HOLM) {
        double mmax = prm->RH_HAGBm0 * std::exp(-1.0 * prm->RH_HAGBHact / (kBoltzmann * T));
        double vmax = mmax * ((Gbhalfsq * rhomax) - pzmin);
        return ((prm->maxfillperstep * prm->cellsize) / vmax);
    }
    double mgs = prm->GSm0 * std::exp(-1.0 * prm->GSHact / (kBoltzmann * T));
    double mhagb = prm->HAGBm0 * std::exp(-1.0 * prm->HAGBHact / (kBoltzmann * T));
    double m_max = (Pmax * mgs) + ((1.0 - Pmax) * mhagb);
    if (Pmax < (0.0 - kDefaultSmallNumber)) m_max = prm->LAGBm0 * std::exp(-1.0 * prm->LAGBHact / (kBoltzmann * T));
    double v_max = m_max * ((Gbhalfsq * rhomax) - pzmin);
    return ((prm->maxfillperstep * prm->cellsize) / v_max);
}

// caHdl::get_dtmax_minimum, SCORE_Kernel.cpp:5687-5723 (the nucleation limit is INFINITE there)
double Physics::dt_minimum() const {
    double m = kInfinite, d;
    d = dt_temp();  if (d < m) m = d;
    d = dt_rho();   if (d < m) m = d;
    d = dt_zener(); if (d < m) m = d;
    d = dt_cells(); if (d < m) m = d;
    return m;
}

// caHdl::update_deformedsubstructure, SCORE_Kernel.cpp:5409-5437 and SCORE_RecoveryModels.cpp:50-126;
// SCORE_RECOVERY_HYPERBOLIC is rho(t) = rho0 / (1 + k t), which the reference does not have.
void Physics::update_substructure(std::vector<double>& rho, const std::vector<double>& rho0) const {
    update_substructure(rho.data(), rho0.data(), 0, rho.size());
}

// grains [lo, n) of the same update (the per-step scalars are recomputed, identically)
void Physics::update_substructure(double* rho, const double* rho0, size_t lo, size_t n) const {
    update_substructure(rho, rho, rho0, lo, n);
}

void Physics::update_substructure(double* rho_out, const double* rho_in, const double* rho0, size_t lo, size_t n) const {
    const int m = prm->recovery_model;
    if (m == SCORE_RECOVERY_NES_VACCOREDIFF) {
        double B = kPi * prm->NesC3 * prm->NesC5 * prm->VacancyDiffD0 * std::exp(-1.0 * prm->VacancyDiffHact / (kBoltzmann * T));
        B /= prm->NesKappa2;
        double exponent = ((b) * (b)) / (kBoltzmann * T);
        double expterm = std::exp(prm->NesAlpha3 * prm->NesKappa2 * G * b * exponent);
        for (size_t g = lo; g < n; ++g) {
            double r_t = 1.0 / std::pow(rho_in[g], 0.5);
            double Bx = (B / r_t) * expterm;
            double r_tdt = (Bx * dt) + r_t;
            rho_out[g] = 1.0 / ((r_tdt) * (r_tdt));
        }
        return;
    }
    if (m == SCORE_RECOVERY_MICHALAKPAXTON) {
        const double f1 = 0.25, f2 = 0.75, tau2 = 0.3605, tau5 = 5.2824;
        double tm = t / 60.0;
        double factor = f1 * std::pow((1 + (tm / tau2)), -1.0) + f2 * std::pow((1 + (tm / tau5)), -0.5);
        for (size_t g = lo; g < n; ++g) rho_out[g] = rho0[g] * ((factor) * (factor));
        return;
    }
    if (m == SCORE_RECOVERY_HYPERBOLIC) {
        double f = 1.0 + prm->recovery_k * t;
        for (size_t g = lo; g < n; ++g) rho_out[g] = rho0[g] / f;
    }
}

double rhomax_of(const std::vector<double>& rho, const std::vector<uint32_t>& counts) {
    double best = -1.0;
    for (size_t g = 0; g < rho.size(); ++g)
        if (counts[g] > 0 && rho[g] > best) best = rho[g];
    return (best >= kRhomaxWellAnnealed) ? best : kRhomaxWellAnnealed;
}

// ---------------------------------------------------------------- .uds reader
// Block format of io::readDataBlock (SCORE_Io.cpp:157-365): a header line
// "|| Name || *(types) ..." then rows of whitespace-separated tokens, one per
// type letter; 's' keeps the string, 'f' parses into a FLOAT (univData.d.f),
// 'i' into an integer.  A row whose first token starts with "||" ends the block;
// blank rows are skipped.

struct UdsRow { std::vector<std::string> s; std::vector<float> f; };
struct UdsBlock { bool found = false; std::string types; std::vector<UdsRow> rows; };

static bool read_block(FILE* fh, const char* wanted, UdsBlock& blk, std::string& err) {
    rewind(fh);
    char buf[1024], name[512], types[512];
    blk = UdsBlock();
    while (fgets(buf, sizeof buf, fh)) {
        char c1 = 0, c2 = 0;
        name[0] = types[0] = 0;
        int cnt = sscanf(buf, "%c%c%511s%*s%511s", &c1, &c2, name, types);
        if (cnt < 3 || c1 != '|' || c2 != '|') continue;
        if (strcmp(name, wanted) != 0) continue;
        if (types[0] != '*' || types[1] != '(') { err = std::string("block header defective: ") + wanted; return false; }
        const char* close = strchr(types + 2, ')');
        if (!close) { err = std::string("block header defective: ") + wanted; return false; }
        blk.types.assign(types + 2, (size_t)(close - (types + 2)));
        blk.found = true;
        break;
    }
    if (!blk.found) { err = std::string("missing block ") + wanted; return false; }
    const size_t ncol = blk.types.size();
    while (fgets(buf, sizeof buf, fh)) {
        UdsRow row;
        size_t pos = 0;
        bool end_block = false, empty = false;
        for (size_t i = 0; i < ncol; ++i) {
            while (buf[pos] == ' ' || buf[pos] == '\t') pos++;
            char tok[1024];
            tok[0] = 0;
            if (sscanf(buf + pos, "%1023s", tok) != 1 || tok[0] == 0) { if (i > 0) { err = std::string("incomplete line in block ") + wanted; return false; } empty = true; break; }
            if (tok[0] == '|' && tok[1] == '|') { if (i > 0) { err = std::string("incomplete line in block ") + wanted; return false; } end_block = true; break; }
            pos += strlen(tok) + 1;
            if (blk.types[i] == 'f') {
                float v;
                if (sscanf(tok, "%f", &v) != 1) { err = std::string("bad number in block ") + wanted; return false; }
                row.f.push_back(v);
                row.s.emplace_back(tok);
            } else {
                row.s.emplace_back(tok);
                row.f.push_back(0.0f);
            }
        }
        if (end_block) break;
        if (empty) continue;
        blk.rows.push_back(row);
    }
    return true;
}

static std::string unquote(std::string s) {
    if (!s.empty() && s[0] == '"') s.erase(0, 1);
    if (!s.empty() && s.back() == '"') s.pop_back();
    return s;
}

static bool get_string(const UdsBlock& b, const char* key, std::string& out) {
    for (const auto& r : b.rows) {
        if (r.s.size() < 2) continue;
        if (unquote(r.s[0]) == key) { out = unquote(r.s[1]); return true; }
    }
    return false;
}

// io::geTReal / io::geTInt (SCORE_Io.cpp:398-426): the whole value must be one number
static bool get_real(const UdsBlock& b, const char* key, double& v, std::string& err) {
    std::string s;
    if (!get_string(b, key, s)) { err = std::string("missing key ") + key; return false; }
    char dummy;
    int cnt = sscanf(s.c_str(), "%lf%c", &v, &dummy);
    if (cnt != 1) { err = std::string("not a double: ") + key; return false; }
    return true;
}
static bool get_int(const UdsBlock& b, const char* key, long& v, std::string& err) {
    std::string s;
    if (!get_string(b, key, s)) { err = std::string("missing key ") + key; return false; }
    char dummy;
    int cnt = sscanf(s.c_str(), "%ld%c", &v, &dummy);
    if (cnt != 1) { err = std::string("not an integer: ") + key; return false; }
    return true;
}

void params_default(score_params* p) {
    memset(p, 0, sizeof *p);
    p->cellsize = 1e-6; p->xmax = 1.0; p->tmax = 360000.0; p->nmax = 1000000;
    p->maxfillperstep = 0.1; p->initial_cache = 0.10; p->recache = 1.0;
    p->mobility_model = SCORE_MOBILITY_SEBALD_GOTTSTEIN;
    p->boundary = SCORE_BOUNDARY_REFERENCE; p->precision = SCORE_PRECISION_FP64;
    p->border_policy = SCORE_BORDER_REFERENCE_LIMIT;
    p->rxarea_threshold = 13;  // log_OUTPUT_Diehl's log_rxareaprofile2( 13 ), SCORE_OnTheFlyCharacterization.cpp:649
}

int uds_read(const char* path, score_params* p, char* errbuf, size_t errlen) {
    std::string err;
    FILE* fh = fopen(path, "r");
    if (!fh) { snprintf(errbuf, errlen, "cannot open %s", path); return SCORE_ERR_IO; }
    params_default(p);
    UdsBlock b;
    long iv = 0;
    double dv = 0;
    bool ok = true;
#define REQ(x) do { if (!(x)) { ok = false; goto done; } } while (0)
    // RuntimeControl, ensembleHdl::init_parameter_runtime (SCORE_Kernel.cpp:262-310)
    REQ(read_block(fh, "RuntimeControl", b, err));
    REQ(get_real(b, "XMAX", p->xmax, err));
    if (p->xmax < 0.0 || p->xmax > 1.0) { err = "invalid XMAX"; ok = false; goto done; }
    REQ(get_real(b, "TIMEMAX", p->tmax, err));
    if (p->tmax < 0.0 || p->tmax > 360000.0) { err = "invalid TIMEMAX"; ok = false; goto done; }
    REQ(get_int(b, "NMAX", iv, err));
    if (iv < 1 || iv > 1000000) { err = "invalid NMAX"; ok = false; goto done; }
    p->nmax = (uint32_t)iv;
    REQ(get_real(b, "MAXFILLPERSTEP", p->maxfillperstep, err));
    if (p->maxfillperstep < 0.01 || p->maxfillperstep > 0.2) p->maxfillperstep = 0.1;
    REQ(get_real(b, "InitialCacheSizeRXCells", p->initial_cache, err));
    if (p->initial_cache < 0.05 || p->initial_cache > 0.25) p->initial_cache = 0.10;
    REQ(get_real(b, "ReCacheSizeRXCells", p->recache, err));
    if (p->recache < 0.5 || p->recache > 2.0) p->recache = 1.0;
    REQ(get_int(b, "OnTheFlyDefragmentation", iv, err));
    p->defragmentation = (iv == 1) ? 1 : 0;
    // EnsembleDefinition, init_parameter_ensemble (SCORE_Kernel.cpp:398-470)
    REQ(read_block(fh, "EnsembleDefinition", b, err));
    REQ(get_real(b, "CellSize", dv, err));
    p->cellsize = dv * 1.0e-6;
    if (p->cellsize < 1e-7 || p->cellsize > 1e-5) { err = "invalid CellSize"; ok = false; goto done; }
    REQ(get_int(b, "3DCAEdgeLengthInCellsRD", iv, err)); p->nx = (uint32_t)iv;
    REQ(get_int(b, "3DCAEdgeLengthInCellsTD", iv, err)); p->ny = (uint32_t)iv;
    REQ(get_int(b, "3DCAEdgeLengthInCellsND", iv, err)); p->nz = (uint32_t)iv;
    // MaterialProperties, init_parameter_material (SCORE_Kernel.cpp:545-562)
    REQ(read_block(fh, "MaterialProperties", b, err));
    REQ(get_real(b, "ZeroKelvinShearModulusG0", p->G0, err));
    REQ(get_real(b, "FirstOrderdG0dT", p->dGdt, err));
    REQ(get_real(b, "ZeroCelsiusBurgersVector", p->bZeroCelsius, err));
    REQ(get_real(b, "MeltingTemperature", dv, err)); p->Tmelt = dv + kToffset;
    // BoundaryMobilityModel, init_parameter_mobilities (SCORE_Kernel.cpp:564-604)
    REQ(read_block(fh, "BoundaryMobilityModel", b, err));
    REQ(get_int(b, "MobilityModel", iv, err));
    p->mobility_model = (iv == 2) ? SCORE_MOBILITY_ROLLETT_HOLM : SCORE_MOBILITY_SEBALD_GOTTSTEIN;
    REQ(get_real(b, "LAGBm0", p->LAGBm0, err));
    REQ(get_real(b, "LAGBHact", dv, err)); p->LAGBHact = dv * kEcharge;
    REQ(get_real(b, "HAGBm0", p->HAGBm0, err));
    REQ(get_real(b, "HAGBHact", dv, err)); p->HAGBHact = dv * kEcharge;
    REQ(get_real(b, "GSm0", p->GSm0, err));
    REQ(get_real(b, "GSHact", dv, err)); p->GSHact = dv * kEcharge;
    REQ(get_real(b, "RHModelHAGBm0", p->RH_HAGBm0, err));
    REQ(get_real(b, "RHModelHAGBHact", dv, err)); p->RH_HAGBHact = dv * kEcharge;
    REQ(get_real(b, "RHModelLAGBHAGBCut", p->RH_cut, err));
    REQ(get_real(b, "RHModelLAGBHAGBTrans", p->RH_trans, err));
    REQ(get_real(b, "RHModelLAGBHAGBExponent", p->RH_exponent, err));
    // RecoveryParameter, init_parameter_recovery (SCORE_Kernel.cpp:606-635)
    REQ(read_block(fh, "RecoveryParameter", b, err));
    REQ(get_int(b, "RecoveryConsider", iv, err));
    p->recovery_model = (iv == 1) ? SCORE_RECOVERY_NES_VACCOREDIFF : (iv == 2) ? SCORE_RECOVERY_NES_SOLUTEDRAG
                      : (iv == 3) ? SCORE_RECOVERY_MICHALAKPAXTON : (iv == 10) ? SCORE_RECOVERY_HYPERBOLIC : SCORE_RECOVERY_NONE;
    REQ(get_real(b, "RecoveryVacancyDiffPreexp", p->VacancyDiffD0, err));
    REQ(get_real(b, "RecoveryVacancyDiffHact", dv, err)); p->VacancyDiffHact = dv * kEcharge;
    REQ(get_real(b, "RecoverySoluteDiffPreexp", p->SoluteDiffD0, err));
    REQ(get_real(b, "RecoverySoluteDiffHact", dv, err)); p->SoluteDiffHact = dv * kEcharge;
    REQ(get_real(b, "RecoverySoluteLsPropFactor", p->SoluteLsPropFactor, err));
    REQ(get_real(b, "RecoverySoluteConcentration", p->SoluteConcentration, err));
    REQ(get_real(b, "RecoveryParameterAlpha3", p->NesAlpha3, err));
    REQ(get_real(b, "RecoveryParameterKappa2", p->NesKappa2, err));
    REQ(get_real(b, "RecoveryParameterC3", p->NesC3, err));
    REQ(get_real(b, "RecoveryParameterC4", p->NesC4, err));
    REQ(get_real(b, "RecoveryParameterC5", p->NesC5, err));
    if (p->recovery_model == SCORE_RECOVERY_HYPERBOLIC) REQ(get_real(b, "RecoveryHyperbolicK", p->recovery_k, err));
    // DragParameter + EvoMicrochemistry, init_parameter_drag (SCORE_Kernel.cpp:637-683)
    REQ(read_block(fh, "DragParameter", b, err));
    REQ(get_int(b, "ZenerConsider", iv, err));
    p->zener_model = (iv == 1) ? SCORE_ZENER_CONSTANT : (iv == 2) ? SCORE_ZENER_TIMEDEP : SCORE_ZENER_NONE;
    REQ(get_real(b, "ZenerAlpha", p->zener_alpha, err));
    REQ(get_real(b, "ZenerGamma", p->zener_gamma, err));
    REQ(read_block(fh, "EvoMicrochemistry", b, err));
    if (b.rows.size() > SCORE_MAX_TABLE) { err = "EvoMicrochemistry too long"; ok = false; goto done; }
    p->n_zener = (uint32_t)b.rows.size();
    for (size_t i = 0; i < b.rows.size(); ++i) {
        if (b.types.size() < 2 || b.types[0] != 'f' || b.types[1] != 'f') { err = "EvoMicrochemistry must be *(ff)"; ok = false; goto done; }
        p->zener_time[i] = (double)b.rows[i].f[0];
        p->zener_fr[i] = (double)b.rows[i].f[1];
    }
    // AnnealingSchedule, init_parameter_processing (SCORE_Kernel.cpp:720-757): float columns, + TOFFSET
    REQ(read_block(fh, "AnnealingSchedule", b, err));
    if (b.rows.size() < 2 || b.rows.size() > SCORE_MAX_TABLE) { err = "AnnealingSchedule needs 2..256 rows"; ok = false; goto done; }
    if (b.types.size() < 2 || b.types[0] != 'f' || b.types[1] != 'f') { err = "AnnealingSchedule must be *(ff)"; ok = false; goto done; }
    p->n_schedule = (uint32_t)b.rows.size();
    {
        double ti_old = -1.0;
        for (size_t i = 0; i < b.rows.size(); ++i) {
            double ti = (double)b.rows[i].f[0];
            double Ti = (double)b.rows[i].f[1];
            Ti += kToffset;
            if (ti < 0.0 || Ti < 0.0 || ti_old >= ti) { err = "invalid annealing schedule"; ok = false; goto done; }
            ti_old = ti;
            p->sched_time[i] = ti;
            p->sched_temp[i] = Ti;
        }
    }
    // HeuristicRXFrontListDefragmentation, init_parameter_additional (SCORE_Kernel.cpp:910-930): column 2, sorted
    REQ(read_block(fh, "HeuristicRXFrontListDefragmentation", b, err));
    if (b.rows.size() > SCORE_MAX_TABLE) { err = "too many defragmentation points"; ok = false; goto done; }
    {
        std::vector<double> xs;
        for (const auto& r : b.rows) {
            if (b.types.size() < 2 || b.types[1] != 'f') { err = "HeuristicRXFrontListDefragmentation column 2 must be f"; ok = false; goto done; }
            double x = (double)r.f[1];
            if (x < 0.0 || x > 1.0) { err = "invalid defragmentation X"; ok = false; goto done; }
            xs.push_back(x);
        }
        std::sort(xs.begin(), xs.end());
        p->n_defrag = (uint32_t)xs.size();
        for (size_t i = 0; i < xs.size(); ++i) p->defrag_x[i] = xs[i];
    }
    // SingleGrainVolOverTime, init_parameter_additional (SCORE_Kernel.cpp:939-957): column 2 (float), sorted
    if (read_block(fh, "SingleGrainVolOverTime", b, err)) {
        if (b.rows.size() > SCORE_MAX_TABLE) { err = "too many SingleGrainVolOverTime logpoints"; ok = false; goto done; }
        std::vector<double> xs;
        for (const auto& r : b.rows) {
            if (b.types.size() < 2 || b.types[1] != 'f') { err = "SingleGrainVolOverTime column 2 must be f"; ok = false; goto done; }
            double x = (double)r.f[1];
            if (x < 0.0 || x > 1.0) { err = "invalid logpoint X"; ok = false; goto done; }
            xs.push_back(x);
        }
        std::sort(xs.begin(), xs.end());
        p->n_logpoints = (uint32_t)xs.size();
        for (size_t i = 0; i < xs.size(); ++i) p->logpoint_x[i] = xs[i];
    }
    err.clear();
    // GB300 build options, optional block "GB300Options" (not part of the reference format)
    if (read_block(fh, "GB300Options", b, err)) {
        if (get_int(b, "Boundary", iv, err)) p->boundary = (int32_t)iv;
        if (get_int(b, "Precision", iv, err)) p->precision = (int32_t)iv;
        if (get_int(b, "BorderPolicy", iv, err)) p->border_policy = (int32_t)iv;
        if (get_int(b, "RXAreaThreshold", iv, err)) p->rxarea_threshold = (uint32_t)iv;
    }
    err.clear();
done:
#undef REQ
    fclose(fh);
    if (!ok) { snprintf(errbuf, errlen, "%s", err.c_str()); return SCORE_ERR_IO; }
    return SCORE_OK;
}

}  // namespace score
