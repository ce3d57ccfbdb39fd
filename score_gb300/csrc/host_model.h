// Host-side FP64 model of the growth step: everything the reference computes on
// its master thread (time, temperature, shear modulus, mobilities, drag,
// recovery, adaptive dt) plus the mobility weight P(rxg,defg).  All expressions
// keep the reference's operation order so results are bit-identical with it when
// compiled without FMA contraction (-ffp-contract=off).
#pragma once
#include <cstdint>
#include <vector>
#include "../../include/score_gb300.h"

namespace score {

// constants, src/SCORE_Defs_Physics.h and src/SCORE_Math.h
constexpr double kBoltzmann = 1.3806488e-23;
constexpr double kToffset = 273.15;
constexpr double kEcharge = 1.602176565e-19;
constexpr double kPi = 3.1415926535897932384626433832795;
constexpr double kRhoRecrystallized = 1.0e11;
constexpr double kDoubleAccuracy = 5.0e-16;
constexpr double kInitialDeltaT = 1e-6;
constexpr double kInfinite = 1e36;
constexpr double kSmallHeatRate = 0.000277777777777777;
constexpr double kSmallRecoveryRate = 2.77e10;
constexpr double kSmallDraggingRate = 0.027777777;
constexpr double kSmallHeat = 1.0;
constexpr double kSmallRho = 1.0e11;
constexpr double kSmallZenerForce = 100.0;
constexpr double kDefaultPmax = 0.0;
constexpr double kRhomaxWellAnnealed = 1e8;
constexpr double kDefaultSmallNumber = 1e-6;
constexpr double kFullRecyclingFactor = 3.0;
constexpr double kRxThreshold = 0.50;
constexpr uint32_t kCurrentlyInfected = 4096002000u;
constexpr double kFgeoFace = 1.0000, kFgeoEdge = 0.7957, kFgeoDiag = 0.6494;
constexpr double kOverFac1 = 0.0682, kOverFac2 = 0.0542, kOverFac3 = 0.0484;

// Mobility weight P of a recrystallized grain (orientation qr) growing into a deformed
// grain (orientation qd): Sebald-Gottstein (-1 LAGB, 0 HAGB, cos^2 near 40deg<111>)
// or Rollett-Holm sigmoid.  Same arithmetic as SCORE_Kernel.cpp:2460-2527.
double mobility_weight(const score_params& p, const double qr[4], const double qd[4]);
// minimum disorientation angle for cubic symmetry, Grimmer's 24 expressions
double disori_angle_cubic(const double p[4], const double q[4]);
// the constants mobility_weight uses, for the device's weight table (no-allocation entry point)
void weight_constants(const score_params& prm, double* fac, double* lagb, double* maxdev, double m40[4], double* theta_sat);
void disori_quat_cubic(const double p[4], const double q[4], double out[4]);

// Scalar state of one domain's growth machine (the caHdl members the master thread updates).
struct Physics {
    const score_params* prm = nullptr;
    double t = 0.0, dt = 0.0, T = 298.15;
    double G = 0.0, b = 0.0, Gbhalfsq = 0.0;
    double mLAGB = 0.0, mHAGB = 0.0, mGS = 0.0, mRHHAGB = 0.0;
    double fr = 0.0, pzmin = 0.0;
    double Pmax = kDefaultPmax;
    double rhomax = kRhomaxWellAnnealed;
    double t_end = 0.0;  // tprocessingend: last annealing-schedule time

    void init(const score_params* p);
    void update_temperature();
    void update_atomistic();
    void update_microchemistry();
    void update_mobilities();
    double zener() const;
    double intrinsic_mobility(double P) const;
    double dt_temp() const;
    double dt_rho() const;
    double dt_zener() const;
    double dt_cells() const;
    double dt_minimum() const;
    // recovery of the per-grain dislocation densities after t += dt
    void update_substructure(std::vector<double>& rho, const std::vector<double>& rho0) const;
    void update_substructure(double* rho, const double* rho0, size_t lo, size_t hi) const;
    // the same update of grains [lo, hi) from rho_in into rho_out (rho_out may be rho_in)
    void update_substructure(double* rho_out, const double* rho_in, const double* rho0, size_t lo, size_t hi) const;
    // driving force p = (Gb^2/2 (rho - rho_rx)) - p_zener, the grow step's inner expression
    double driving_force(double rho) const;
};

// max rho over grains that still have cells, floored at the well-annealed value
// (update_myrhomax, SCORE_RecoveryModels.cpp:150-170)
double rhomax_of(const std::vector<double>& rho, const std::vector<uint32_t>& counts);

int uds_read(const char* path, score_params* out, char* err, size_t errlen);
void params_default(score_params* out);

}  // namespace score
