// Synthetic deformed structures: the periodic Voronoi grid shared by the host generator
// (host_generate.cpp) and its device fill (synthesis.cu).
#pragma once
#include <cstdint>
#include <functional>
#include <vector>

#include "../../include/score_gb300.h"

namespace score {

// Seeds binned into nb[0] x nb[1] x nb[2] buckets of width bw (cells) per axis; the seeds of bucket b
// are items[start[b] .. start[b + 1]) in ascending id.  Distance: d^2 = sum (periodic |dx_a| / scale_a)^2.
struct VoronoiGrid {
    uint32_t n[3];
    double scale[3];
    std::vector<double> pos;        // 3 per seed
    uint32_t nb[3];
    double bw[3];
    std::vector<uint32_t> start, items;
};

// score_generate_domain with the label fill replaced by `fill` (same seeds, same RNG stream)
int generate_domain_with(const score_gen_params* g, uint32_t* grid, double* defg_quat, double* defg_rho0, double* rxg_quat,
                         uint32_t* rxg_site, double* rxg_tincub, const std::function<int(const VoronoiGrid&, uint32_t*)>& fill);
int fill_voronoi_host(const VoronoiGrid& vg, uint32_t* grid);

}  // namespace score
