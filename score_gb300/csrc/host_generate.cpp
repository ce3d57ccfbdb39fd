// Deterministic synthetic domains for the growth step (test and benchmark inputs).
//
// Every value is produced with integer arithmetic and IEEE basic operations only
// (+ - * / sqrt, floor, frexp, ldexp), never libm transcendentals, so x86-64 and
// aarch64 hosts produce identical bits.  Compiled with -ffp-contract=off.
//
//   deformed grains : periodic Voronoi of `ngrains` uniform seeds, optional per-axis
//                     metric scale (aspect 1:4:8 gives rolled "pancake" grains)
//   orientations    : uniform on SO(3) (normalised 4-ball rejection sample) or clustered
//                     around `ncomp` random texture components with Gaussian scatter
//   dislocation rho : lognormal (mean, sigma of ln rho) or bimodal lo/hi 50/50
//   nuclei          : distinct sites in draw order; uniform, or a fraction forced onto
//                     grain-boundary cells; orientation uniform; Poisson incubation times
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_set>
#include <vector>
#include <algorithm>
#include <functional>
#include "../../include/score_gb300.h"
#include "host_generate.h"

namespace {

struct Rng {  // xoshiro256** seeded by splitmix64
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (int i = 0; i < 4; ++i) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            s[i] = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double u01() { return (double)(next() >> 11) * 0x1.0p-53; }   // [0,1)
    uint64_t below(uint64_t n) {                                    // unbiased [0,n)
        uint64_t lim = ~0ull - (~0ull % n);
        uint64_t x;
        do { x = next(); } while (x >= lim);
        return x % n;
    }
};

// natural log from frexp + atanh series (deterministic, ~1 ulp)
double det_log(double x) {
    int e;
    double m = std::frexp(x, &e);  // x = m 2^e, m in [0.5,1)
    if (m < 0.70710678118654752) { m *= 2.0; e -= 1; }
    double s = (m - 1.0) / (m + 1.0), s2 = s * s, term = s, sum = 0.0;
    for (int k = 1; k < 40; k += 2) { sum += term / k; term *= s2; }
    const double ln2_hi = 0.693147180369123816490, ln2_lo = 1.90821492927058770002e-10;
    return (double)e * ln2_hi + (2.0 * sum + (double)e * ln2_lo);
}
// exp by ln2 range reduction + Taylor series (deterministic, ~1 ulp)
double det_exp(double x) {
    const double ln2_hi = 0.693147180369123816490, ln2_lo = 1.90821492927058770002e-10;
    double k = std::floor(x / 0.69314718055994530942 + 0.5);
    double r = (x - k * ln2_hi) - k * ln2_lo;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 25; ++i) { term = term * r / i; sum += term; }
    return std::ldexp(sum, (int)k);
}
// standard normal by the Marsaglia polar method
double det_normal(Rng& g) {
    for (;;) {
        double u = 2.0 * g.u01() - 1.0, v = 2.0 * g.u01() - 1.0, s = u * u + v * v;
        if (s > 0.0 && s < 1.0) return u * std::sqrt(-2.0 * det_log(s) / s);
    }
}
// uniform random rotation: normalised point uniform in the unit 4-ball
void det_quat(Rng& g, double q[4]) {
    for (;;) {
        double a = 2.0 * g.u01() - 1.0, b = 2.0 * g.u01() - 1.0, c = 2.0 * g.u01() - 1.0, d = 2.0 * g.u01() - 1.0;
        double n2 = a * a + b * b + c * c + d * d;
        if (n2 > 1e-6 && n2 <= 1.0) {
            double n = std::sqrt(n2);
            q[0] = a / n; q[1] = b / n; q[2] = c / n; q[3] = d / n;
            if (q[0] < 0) { q[0] = -q[0]; q[1] = -q[1]; q[2] = -q[2]; q[3] = -q[3]; }
            return;
        }
    }
}
// small rotation with angle |N(0,sigma)| about a uniform axis, applied to q
void det_scatter(Rng& g, const double q[4], double sigma_rad, double out[4]) {
    double ax[3];
    for (;;) {
        ax[0] = 2.0 * g.u01() - 1.0; ax[1] = 2.0 * g.u01() - 1.0; ax[2] = 2.0 * g.u01() - 1.0;
        double n2 = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
        if (n2 > 1e-6 && n2 <= 1.0) { double n = std::sqrt(n2); ax[0] /= n; ax[1] /= n; ax[2] /= n; break; }
    }
    double w = sigma_rad * det_normal(g);
    // half-angle sine/cosine by Taylor series (|w/2| is small)
    double h = 0.5 * w, h2 = h * h, s = 0.0, c = 0.0, ts = h, tc = 1.0;
    for (int k = 0; k < 20; ++k) {
        s += ts; c += tc;
        ts = -ts * h2 / ((2 * k + 2) * (2 * k + 3));
        tc = -tc * h2 / ((2 * k + 1) * (2 * k + 2));
    }
    double r[4] = {c, s * ax[0], s * ax[1], s * ax[2]};
    out[0] = r[0] * q[0] - r[1] * q[1] - r[2] * q[2] - r[3] * q[3];
    out[1] = r[0] * q[1] + r[1] * q[0] + r[2] * q[3] - r[3] * q[2];
    out[2] = r[0] * q[2] - r[1] * q[3] + r[2] * q[0] + r[3] * q[1];
    out[3] = r[0] * q[3] + r[1] * q[2] - r[2] * q[1] + r[3] * q[0];
    double n = std::sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2] + out[3] * out[3]);
    for (int i = 0; i < 4; ++i) out[i] /= n;
}

struct Voronoi : score::VoronoiGrid {

    void build() {
        const size_t S = pos.size() / 3;
        double vol = (double)n[0] * n[1] * n[2];
        double spacing = std::cbrt(vol / (double)S);
        for (int a = 0; a < 3; ++a) {
            double w = spacing * scale[a] / std::cbrt(scale[0] * scale[1] * scale[2]);
            uint32_t k = (uint32_t)std::max(1.0, std::floor((double)n[a] / std::max(1.0, w)));
            nb[a] = k; bw[a] = (double)n[a] / k;
        }
        size_t NB = (size_t)nb[0] * nb[1] * nb[2];
        std::vector<uint32_t> cnt(NB + 1, 0);
        std::vector<uint32_t> home(S);
        for (size_t s = 0; s < S; ++s) {
            uint32_t b[3];
            for (int a = 0; a < 3; ++a) { b[a] = (uint32_t)(pos[3 * s + a] / bw[a]); if (b[a] >= nb[a]) b[a] = nb[a] - 1; }
            home[s] = b[0] + nb[0] * (b[1] + nb[1] * b[2]);
            cnt[home[s] + 1]++;
        }
        for (size_t i = 0; i < NB; ++i) cnt[i + 1] += cnt[i];
        start = cnt;
        items.assign(S, 0);
        std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
        for (size_t s = 0; s < S; ++s) items[fill[home[s]]++] = (uint32_t)s;  // ascending seed id per bucket
    }

    inline double d2(uint32_t s, const double c[3]) const {
        double r = 0.0;
        for (int a = 0; a < 3; ++a) {
            double d = std::fabs(c[a] - pos[3 * s + a]);
            double e = (double)n[a] - d;
            if (e < d) d = e;
            d = d / scale[a];
            r += d * d;
        }
        return r;
    }

    // nearest seed (ties -> lowest id) of the cell centre (x+0.5, y+0.5, z+0.5)
    uint32_t nearest(uint32_t x, uint32_t y, uint32_t z) const {
        const double c[3] = {x + 0.5, y + 0.5, z + 0.5};
        int home[3] = {(int)(c[0] / bw[0]), (int)(c[1] / bw[1]), (int)(c[2] / bw[2])};
        for (int a = 0; a < 3; ++a) if (home[a] >= (int)nb[a]) home[a] = nb[a] - 1;
        double best = 1e300;
        uint32_t arg = 0xFFFFFFFFu;
        int maxr = (int)std::max(nb[0], std::max(nb[1], nb[2]));
        for (int r = 0; r <= maxr; ++r) {
            // visit the shell of Chebyshev radius r (buckets wrap periodically)
            for (int dz = -r; dz <= r; ++dz)
                for (int dy = -r; dy <= r; ++dy)
                    for (int dx = -r; dx <= r; ++dx) {
                        if (std::max(std::abs(dx), std::max(std::abs(dy), std::abs(dz))) != r) continue;
                        int bx = ((home[0] + dx) % (int)nb[0] + (int)nb[0]) % (int)nb[0];
                        int by = ((home[1] + dy) % (int)nb[1] + (int)nb[1]) % (int)nb[1];
                        int bz = ((home[2] + dz) % (int)nb[2] + (int)nb[2]) % (int)nb[2];
                        uint32_t b = bx + nb[0] * (by + nb[1] * bz);
                        for (uint32_t i = start[b]; i < start[b + 1]; ++i) {
                            uint32_t s = items[i];
                            double v = d2(s, c);
                            if (v < best || (v == best && s < arg)) { best = v; arg = s; }
                        }
                    }
            // every unvisited bucket is at least r bucket widths away along some axis
            double lb = 1e300;
            for (int a = 0; a < 3; ++a) lb = std::min(lb, (double)r * bw[a] / scale[a]);
            if (arg != 0xFFFFFFFFu && best <= lb * lb) break;
        }
        return arg;
    }
};

}  // namespace

namespace score {

// Host fill: every cell's nearest seed, z slabs spread over the host threads.
int fill_voronoi_host(const VoronoiGrid& vg, uint32_t* grid) {
    const Voronoi& vo = static_cast<const Voronoi&>(vg);
    unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t)
        th.emplace_back([&, t]() {
            for (uint32_t z = t; z < vo.n[2]; z += nth)
                for (uint32_t y = 0; y < vo.n[1]; ++y)
                    for (uint32_t x = 0; x < vo.n[0]; ++x)
                        grid[(size_t)x + (size_t)vo.n[0] * (y + (size_t)vo.n[1] * z)] = vo.nearest(x, y, z);
        });
    for (auto& t : th) t.join();
    return SCORE_OK;
}

}  // namespace score

extern "C" int score_gen_default(score_gen_params* g) {
    if (!g) return SCORE_ERR_ARG;
    memset(g, 0, sizeof *g);
    g->nx = g->ny = g->nz = 128;
    g->ngrains = 500; g->nnuclei = 200; g->seed = 0;
    g->rho_mean = 1e15; g->rho_sigma = 0.3; g->rho_mode = 0;
    g->rho_lo = 1e14; g->rho_hi = 5e15;
    g->aspect[0] = g->aspect[1] = g->aspect[2] = 1.0;
    g->ori_mode = 0; g->ncomp = 3; g->scatter_deg = 10.0;
    g->site_mode = 0; g->gb_fraction = 0.8; g->nucleation_rate = 0.0;
    return SCORE_OK;
}

namespace score {

int generate_domain_with(const score_gen_params* g, uint32_t* grid, double* defg_quat, double* defg_rho0, double* rxg_quat,
                         uint32_t* rxg_site, double* rxg_tincub, const std::function<int(const VoronoiGrid&, uint32_t*)>& fill) {
    if (!g || !grid || !defg_quat || !defg_rho0 || !rxg_quat || !rxg_site) return SCORE_ERR_ARG;
    if (g->nx == 0 || g->ny == 0 || g->nz == 0 || g->ngrains == 0) return SCORE_ERR_ARG;
    const uint64_t N = (uint64_t)g->nx * g->ny * g->nz;
    if (N > 0xFFFFFFFFull || g->nnuclei > N) return SCORE_ERR_ARG;
    Rng rng(g->seed * 0x9E3779B97F4A7C15ull + 0x1234567ull);

    // 1) Voronoi seeds and labels
    Voronoi vo;
    vo.n[0] = g->nx; vo.n[1] = g->ny; vo.n[2] = g->nz;
    for (int a = 0; a < 3; ++a) vo.scale[a] = g->aspect[a] > 0 ? g->aspect[a] : 1.0;
    vo.pos.resize((size_t)g->ngrains * 3);
    for (uint32_t s = 0; s < g->ngrains; ++s) {
        vo.pos[3 * s + 0] = rng.u01() * g->nx;
        vo.pos[3 * s + 1] = rng.u01() * g->ny;
        vo.pos[3 * s + 2] = rng.u01() * g->nz;
    }
    vo.build();
    const int fs = fill(vo, grid);  // the seed pass is the only RNG use before the fill
    if (fs != SCORE_OK) return fs;

    // 2) grain orientations and dislocation densities
    std::vector<double> comps((size_t)std::max(1u, g->ncomp) * 4);
    for (uint32_t c = 0; c < std::max(1u, g->ncomp); ++c) det_quat(rng, &comps[4 * c]);
    const double sigma_rad = g->scatter_deg / 180.0 * 3.14159265358979323846;
    const double mu = det_log(g->rho_mean) - 0.5 * g->rho_sigma * g->rho_sigma;
    for (uint32_t s = 0; s < g->ngrains; ++s) {
        if (g->ori_mode == 1) det_scatter(rng, &comps[4 * rng.below(std::max(1u, g->ncomp))], sigma_rad, &defg_quat[4 * (size_t)s]);
        else det_quat(rng, &defg_quat[4 * (size_t)s]);
        if (g->rho_mode == 1) defg_rho0[s] = (rng.next() >> 63) ? g->rho_hi : g->rho_lo;
        else defg_rho0[s] = det_exp(mu + g->rho_sigma * det_normal(rng));
    }

    // 3) nucleation sites (distinct, draw order) and orientations
    std::unordered_set<uint32_t> used;
    used.reserve((size_t)g->nnuclei * 2);
    const uint32_t nx = g->nx, ny = g->ny, nz = g->nz;
    auto on_boundary = [&](uint32_t idx) {
        uint32_t x = idx % nx, y = (idx / nx) % ny, z = idx / (nx * ny);
        uint32_t me = grid[idx];
        const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        for (auto& o : off) {
            uint32_t xx = (x + nx + o[0]) % nx, yy = (y + ny + o[1]) % ny, zz = (z + nz + o[2]) % nz;
            if (grid[(size_t)xx + (size_t)nx * (yy + (size_t)ny * zz)] != me) return true;
        }
        return false;
    };
    double tnow = 0.0;
    for (uint32_t k = 0; k < g->nnuclei; ++k) {
        bool want_gb = (g->site_mode == 1) && (rng.u01() < g->gb_fraction);
        uint32_t site;
        for (int attempt = 0;; ++attempt) {
            site = (uint32_t)rng.below(N);
            if (used.count(site)) continue;
            if (want_gb && attempt < 100000 && !on_boundary(site)) continue;
            break;
        }
        used.insert(site);
        rxg_site[k] = site;
        det_quat(rng, &rxg_quat[4 * (size_t)k]);
        if (rxg_tincub) {
            if (g->nucleation_rate > 0.0) { tnow += -det_log(1.0 - rng.u01()) / g->nucleation_rate; rxg_tincub[k] = tnow; }
            else rxg_tincub[k] = 0.0;
        }
    }
    return SCORE_OK;
}

}  // namespace score

extern "C" int score_generate_domain(const score_gen_params* g, uint32_t* grid, double* defg_quat, double* defg_rho0,
                                     double* rxg_quat, uint32_t* rxg_site, double* rxg_tincub) {
    return score::generate_domain_with(g, grid, defg_quat, defg_rho0, rxg_quat, rxg_site, rxg_tincub, score::fill_voronoi_host);
}
