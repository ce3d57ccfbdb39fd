// Deformed-structure synthesis on the device: the periodic Voronoi label fill of the synthetic
// domains (host_generate.cpp) as a CUDA kernel, bit for bit the host's labels.
//
// Each thread labels one cell with its nearest seed (ties to the lowest id) by the host's bucket
// search: shells of Chebyshev radius r around the cell's home bucket, visited until the nearest
// distance found is within the lower bound r bw / scale of every unvisited bucket.  Distances use
// the host's FP64 operation sequence (periodic |dx|, division by the metric scale, square, sum;
// no contraction into FMA: this file is compiled with -fmad=false), so every comparison, and hence
// every label, is the host's.  The seeds, orientations, densities and nuclei stay on the host's
// random stream; the fill consumes no random numbers.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/score_gb300.h"
#include "host_generate.h"

namespace {

struct VoronoiDev {
    uint32_t n[3], nb[3];
    double scale[3], bw[3];
    int unit_scale;                 // every scale is 1: the division is skipped (x / 1.0 == x)
    const double* pos;
    const uint32_t* start;
    const uint32_t* items;
};

__device__ __forceinline__ double seed_d2(const VoronoiDev& v, uint32_t s, const double c[3]) {
    double r = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double d = fabs(__dsub_rn(c[a], __ldg(&v.pos[3 * s + a])));
        const double e = __dsub_rn((double)v.n[a], d);
        if (e < d) d = e;
        if (!v.unit_scale) d = __ddiv_rn(d, v.scale[a]);
        r = __dadd_rn(r, __dmul_rn(d, d));
    }
    return r;
}

__global__ void __launch_bounds__(256) k_voronoi_fill(VoronoiDev v, uint32_t* grid) {
    const uint64_t N = (uint64_t)v.n[0] * v.n[1] * v.n[2];
    const int nbx = (int)v.nb[0], nby = (int)v.nb[1], nbz = (int)v.nb[2];
    const int maxr = max(nbx, max(nby, nbz));
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(i % v.n[0]), y = (uint32_t)((i / v.n[0]) % v.n[1]), z = (uint32_t)(i / ((uint64_t)v.n[0] * v.n[1]));
        const double c[3] = {x + 0.5, y + 0.5, z + 0.5};
        int home[3] = {(int)__ddiv_rn(c[0], v.bw[0]), (int)__ddiv_rn(c[1], v.bw[1]), (int)__ddiv_rn(c[2], v.bw[2])};
        if (home[0] >= nbx) home[0] = nbx - 1;
        if (home[1] >= nby) home[1] = nby - 1;
        if (home[2] >= nbz) home[2] = nbz - 1;
        double best = 1e300;
        uint32_t arg = 0xFFFFFFFFu;
        for (int r = 0; r <= maxr; ++r) {
            for (int dz = -r; dz <= r; ++dz)
                for (int dy = -r; dy <= r; ++dy)
                    for (int dx = -r; dx <= r; ++dx) {
                        if (max(abs(dx), max(abs(dy), abs(dz))) != r) continue;
                        const int bx = ((home[0] + dx) % nbx + nbx) % nbx;
                        const int by = ((home[1] + dy) % nby + nby) % nby;
                        const int bz = ((home[2] + dz) % nbz + nbz) % nbz;
                        const uint32_t b = (uint32_t)bx + v.nb[0] * ((uint32_t)by + v.nb[1] * (uint32_t)bz);
                        const uint32_t e = __ldg(&v.start[b + 1]);
                        for (uint32_t k = __ldg(&v.start[b]); k < e; ++k) {
                            const uint32_t s = __ldg(&v.items[k]);
                            const double d = seed_d2(v, s, c);
                            if (d < best || (d == best && s < arg)) { best = d; arg = s; }
                        }
                    }
            double lb = 1e300;
#pragma unroll
            for (int a = 0; a < 3; ++a) lb = fmin(lb, __ddiv_rn(__dmul_rn((double)r, v.bw[a]), v.scale[a]));
            if (arg != 0xFFFFFFFFu && best <= __dmul_rn(lb, lb)) break;
        }
        grid[i] = arg;
    }
}

// The device fill behind score_generate_domain_gpu; the labels go back to the host grid.
int fill_voronoi_device(const score::VoronoiGrid& vg, uint32_t* grid, int device, std::string& err) {
    const uint64_t N = (uint64_t)vg.n[0] * vg.n[1] * vg.n[2];
    const size_t S = vg.pos.size() / 3, NB = vg.start.size();
    cudaError_t e = cudaSetDevice(device);
    int sms = 1;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    char* blk = nullptr;
    const size_t b_pos = ((S * 3 * 8) + 255) & ~(size_t)255, b_st = ((NB * 4) + 255) & ~(size_t)255, b_it = ((S * 4) + 255) & ~(size_t)255;
    if (e == cudaSuccess) e = cudaMalloc((void**)&blk, b_pos + b_st + b_it + N * 4);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return SCORE_ERR_NOMEM; }
    VoronoiDev v{};
    for (int a = 0; a < 3; ++a) { v.n[a] = vg.n[a]; v.nb[a] = vg.nb[a]; v.scale[a] = vg.scale[a]; v.bw[a] = vg.bw[a]; }
    v.unit_scale = vg.scale[0] == 1.0 && vg.scale[1] == 1.0 && vg.scale[2] == 1.0;
    v.pos = (const double*)blk;
    v.start = (const uint32_t*)(blk + b_pos);
    v.items = (const uint32_t*)(blk + b_pos + b_st);
    uint32_t* d_grid = (uint32_t*)(blk + b_pos + b_st + b_it);
    e = cudaMemcpy((void*)v.pos, vg.pos.data(), S * 3 * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy((void*)v.start, vg.start.data(), NB * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy((void*)v.items, vg.items.data(), S * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_voronoi_fill<<<(unsigned)sms * 8, 256>>>(v, d_grid);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(grid, d_grid, N * 4, cudaMemcpyDeviceToHost);
    cudaFree(blk);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return SCORE_ERR_CUDA; }
    return SCORE_OK;
}

}  // namespace

extern "C" int score_generate_domain_gpu(const score_gen_params* g, uint32_t* grid, double* defg_quat, double* defg_rho0,
                                         double* rxg_quat, uint32_t* rxg_site, double* rxg_tincub, int device) {
    if (!g) return SCORE_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return SCORE_ERR_NOT_BUILT; }
    if (device < 0 || device >= ndev) return SCORE_ERR_ARG;
    std::string err;
    return score::generate_domain_with(g, grid, defg_quat, defg_rho0, rxg_quat, rxg_site, rxg_tincub,
                                       [&](const score::VoronoiGrid& vg, uint32_t* out) { return fill_voronoi_device(vg, out, device, err); });
}
