// Percolation analysis on the device: the clusters of recrystallized and infected cells
// (caHdl::log_PERCOLATION, SCORE_OnTheFlyCharacterization.cpp:777-875, and its percAnalyzer,
// SCORE_PercAnalyzer.cpp), as a parallel union-find instead of the reference's sequential
// Hoshen-Kopelman scan.
//
// The scan's union-find ends with the connected components of the links it makes, and every link
// is decided by the cell and its three lower neighbours alone (hk3d_core_nonperiodic, :161-226): a
// cell links to each lower neighbour (-x, -y, -z) that is a 1-cell other than the origin (labels are
// cell indices and 0 means "not recrystallized", so the origin never joins a cluster), except that
// with all three present it links to the lower y and z neighbours only (:218-225).  So the
// reference's clusters are found exactly by linking those pairs in any order (SCORE_PERC_REFERENCE);
// SCORE_PERC_CONNECTED links all present lower neighbours: the true 6-connected clusters.
//
// Kernels: init (parent = self for 1-cells), link (lock-free union: the larger root is attached to
// the smaller with atomicCAS, path halving in find), flatten (read-only walks), then the compaction of
// compactify (:334-390): clusters numbered in the order of their first cell, which is the root (the
// smallest index of a cluster) order, by a count / scan / assign pass; then per-cluster sizes and face
// bits for percolates (:500-615) and the size distribution (:617-656, sorted on the host).
#include "percolation.h"

#include <algorithm>
#include <vector>

namespace score {
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kPercTile = 2048;          // cells per count / assign tile (256 threads x 8)
constexpr uint32_t kFindLimit = 1u << 24;     // bounded pointer chasing: a longer chain flags an error
constexpr uint32_t kUniteLimit = 1u << 20;    // bounded link retries

__device__ __forceinline__ bool is_one(const uint32_t* grid, uint64_t c, uint32_t ndefg) { return c != 0 && grid[c] >= ndefg; }

__device__ __forceinline__ uint32_t find_root(uint32_t* parent, uint32_t x, uint32_t* err) {
    for (uint32_t k = 0; k < kFindLimit; ++k) {
        const uint32_t p = parent[x];
        if (p == x) return x;
        const uint32_t g = parent[p];
        if (g != p) parent[x] = g;  // path halving: g is an ancestor of x, any interleaving keeps the forest
        x = p;
    }
    atomicOr(err, 1u);
    return x;
}

__device__ __forceinline__ void unite(uint32_t* parent, uint32_t a, uint32_t b, uint32_t* err) {
    for (uint32_t k = 0; k < kUniteLimit; ++k) {
        a = find_root(parent, a, err);
        b = find_root(parent, b, err);
        if (a == b) return;
        if (a < b) { const uint32_t t = a; a = b; b = t; }
        const uint32_t old = atomicCAS(&parent[a], a, b);  // attach the larger root below the smaller
        if (old == a) return;
        a = old;  // a was attached elsewhere meanwhile: retry from its new parent
    }
    atomicOr(err, 2u);
}

__global__ void k_perc_init(const uint32_t* grid, uint64_t N, uint32_t ndefg, uint32_t* parent) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x)
        parent[i] = is_one(grid, i, ndefg) ? (uint32_t)i : kNone;
}

__global__ void k_perc_link(const uint32_t* grid, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t ndefg, int mode, uint32_t* parent,
                            uint32_t* err) {
    const uint64_t nxy = (uint64_t)nx * ny, N = nxy * nz;
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < N; c += (uint64_t)gridDim.x * blockDim.x) {
        if (!is_one(grid, c, ndefg)) continue;
        const uint32_t x = (uint32_t)(c % nx), y = (uint32_t)((c / nx) % ny), z = (uint32_t)(c / nxy);
        const bool l = x > 0 && is_one(grid, c - 1, ndefg);
        const bool b = y > 0 && is_one(grid, c - nx, ndefg);
        const bool f = z > 0 && is_one(grid, c - nxy, ndefg);
        if (l && !(mode == SCORE_PERC_REFERENCE && b && f)) unite(parent, (uint32_t)c, (uint32_t)(c - 1), err);
        if (b) unite(parent, (uint32_t)c, (uint32_t)(c - nx), err);
        if (f) unite(parent, (uint32_t)c, (uint32_t)(c - nxy), err);
    }
}

// Every cell's root.  The walk only reads: path halving here could overwrite the root another
// thread just stored for its own cell with an older ancestor, and the labels read parent as the root.
// Concurrent stores of other cells' roots only shorten the paths walked.
__global__ void k_perc_flatten(uint32_t* parent, uint64_t N, uint32_t* err) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = parent[i];
        if (x == kNone) continue;
        uint32_t k = 0;
        for (uint32_t p = parent[x]; p != x && k < kFindLimit; p = parent[x], ++k) x = p;
        if (k == kFindLimit) atomicOr(err, 1u);
        parent[i] = x;
    }
}

// roots per tile of kPercTile cells (a root is a cell that is its own parent)
__global__ void __launch_bounds__(256) k_perc_count(const uint32_t* parent, uint64_t N, uint32_t* tilecnt) {
    __shared__ uint32_t s_w[8];
    const uint64_t t0 = (uint64_t)blockIdx.x * kPercTile;
    uint32_t c = 0;
    for (uint32_t k = threadIdx.x; k < kPercTile; k += 256) {
        const uint64_t i = t0 + k;
        c += (i < N && parent[i] == (uint32_t)i) ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; ++w) t += s_w[w];
        tilecnt[blockIdx.x] = t;
    }
}

// exclusive scan of the tile counts by one block; total in *total
__global__ void __launch_bounds__(1024) k_perc_scan(uint32_t* tilecnt, uint32_t ntiles, uint32_t* total) {
    __shared__ uint32_t s_w[32], s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < ntiles; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < ntiles ? tilecnt[i] : 0u;
        uint32_t inc = v;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += x;
        }
        if (lane == 31) s_w[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w += x;
            }
            s_w[lane] = w;
        }
        __syncthreads();
        if (i < ntiles) tilecnt[i] = s_carry + (warp ? s_w[warp - 1] : 0u) + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_w[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = s_carry;
}

// compact label of every root: 1 + roots before it (the reference's order of first appearance)
__global__ void __launch_bounds__(256) k_perc_assign(const uint32_t* parent, uint64_t N, const uint32_t* tilebase, uint32_t* cid) {
    __shared__ uint32_t s_w[8], s_run;
    const uint64_t t0 = (uint64_t)blockIdx.x * kPercTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_run = tilebase[blockIdx.x];
    __syncthreads();
    for (uint32_t k0 = 0; k0 < kPercTile; k0 += 256) {
        const uint64_t i = t0 + k0 + threadIdx.x;
        const bool root = i < N && parent[i] == (uint32_t)i;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, root);
        if (lane == 0) s_w[warp] = __popc(m);
        __syncthreads();
        uint32_t before = s_run;
        for (int w = 0; w < warp; ++w) before += s_w[w];
        if (root) cid[i] = before + (uint32_t)__popc(m & ((1u << lane) - 1u)) + 1u;
        __syncthreads();
        if (threadIdx.x == 0) for (int w = 0; w < 8; ++w) s_run += s_w[w];
        __syncthreads();
    }
}

// every cell's compact label, cluster sizes and face bits (cells of one warp in one cluster add together)
__global__ void k_perc_label(const uint32_t* parent, const uint32_t* cid, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t* label,
                             uint32_t* size, uint32_t* face) {
    const uint64_t nxy = (uint64_t)nx * ny, N = nxy * nz;
    const uint64_t end = (N + 31) & ~31ull;
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < end; c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t l = 0, bits = 0;
        if (c < N) {
            const uint32_t p = parent[c];
            if (p != kNone) {
                l = cid[p];
                const uint32_t x = (uint32_t)(c % nx), y = (uint32_t)((c / nx) % ny), z = (uint32_t)(c / nxy);
                bits = (x == 0 ? 1u : 0u) | (x == nx - 1 ? 2u : 0u) | (y == 0 ? 4u : 0u) | (y == ny - 1 ? 8u : 0u) |
                       (z == 0 ? 16u : 0u) | (z == nz - 1 ? 32u : 0u);
            }
            label[c] = l;
        }
        const uint32_t m = __match_any_sync(0xFFFFFFFFu, l);
        uint32_t b = bits;
        for (uint32_t mm = m; mm; mm &= mm - 1) b |= __shfl_sync(m, bits, __ffs(mm) - 1);
        if (l && (__ffs(m) - 1) == (int)(threadIdx.x & 31)) {
            atomicAdd(&size[l - 1], (uint32_t)__popc(m));
            if (b) atomicOr(&face[l - 1], b);
        }
    }
}

}  // namespace

int percolation_analyze(const uint32_t* grid, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t ndefg, int mode, cudaStream_t st,
                        int sms, score_perc_result* out, uint32_t* sizes, uint32_t sizes_cap, uint32_t* labels, std::string& err) {
    if (mode != SCORE_PERC_REFERENCE && mode != SCORE_PERC_CONNECTED) { err = "unknown percolation mode"; return SCORE_ERR_ARG; }
    const uint64_t N = (uint64_t)nx * ny * nz;
    const uint32_t ntiles = (uint32_t)((N + kPercTile - 1) / kPercTile);
    const uint64_t maxc = N / 2 + 2;  // at most every other cell of a 6-connected structure starts a cluster
    auto up = [](uint64_t x) { return (x + 255) & ~(uint64_t)255; };
    const uint64_t b_par = up(N * 4), b_cid = up(N * 4), b_lab = up(N * 4), b_sz = up(maxc * 4), b_fc = up(maxc * 4),
                   b_tile = up((uint64_t)ntiles * 4), b_misc = 256;
    char* blk = nullptr;
    cudaError_t e = cudaMalloc((void**)&blk, b_par + b_cid + b_lab + b_sz + b_fc + b_tile + b_misc);
    if (e != cudaSuccess) { err = "percolation buffers"; return SCORE_ERR_NOMEM; }
    uint32_t* parent = (uint32_t*)blk;
    uint32_t* cid = (uint32_t*)(blk + b_par);
    uint32_t* lab = (uint32_t*)(blk + b_par + b_cid);
    uint32_t* size = (uint32_t*)(blk + b_par + b_cid + b_lab);
    uint32_t* face = (uint32_t*)(blk + b_par + b_cid + b_lab + b_sz);
    uint32_t* tile = (uint32_t*)(blk + b_par + b_cid + b_lab + b_sz + b_fc);
    uint32_t* misc = (uint32_t*)(blk + b_par + b_cid + b_lab + b_sz + b_fc + b_tile);  // [0] total, [1] error flags
    const uint32_t g = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((N + 255) / 256, (uint64_t)sms * 16));
    e = cudaMemsetAsync(misc, 0, 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(size, 0, maxc * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(face, 0, maxc * 4, st);
    if (e == cudaSuccess) {
        k_perc_init<<<g, 256, 0, st>>>(grid, N, ndefg, parent);
        k_perc_link<<<g, 256, 0, st>>>(grid, nx, ny, nz, ndefg, mode, parent, misc + 1);
        k_perc_flatten<<<g, 256, 0, st>>>(parent, N, misc + 1);
        k_perc_count<<<ntiles, 256, 0, st>>>(parent, N, tile);
        k_perc_scan<<<1, 1024, 0, st>>>(tile, ntiles, misc);
        k_perc_assign<<<ntiles, 256, 0, st>>>(parent, N, tile, cid);
        k_perc_label<<<g, 256, 0, st>>>(parent, cid, nx, ny, nz, lab, size, face);
        e = cudaGetLastError();
    }
    uint32_t hm[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm, misc, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    std::vector<uint32_t> hs, hf;
    if (e == cudaSuccess && hm[1] == 0) {
        hs.resize(hm[0]);
        hf.resize(hm[0]);
        if (hm[0]) e = cudaMemcpyAsync(hs.data(), size, (size_t)hm[0] * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && hm[0]) e = cudaMemcpyAsync(hf.data(), face, (size_t)hm[0] * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && labels) e = cudaMemcpyAsync(labels, lab, N * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(blk);
    if (e != cudaSuccess) { err = std::string("percolation: ") + cudaGetErrorString(e); return SCORE_ERR_CUDA; }
    if (hm[1]) { err = "percolation: a bounded union-find loop gave up"; return SCORE_ERR_TIMEOUT; }
    score_perc_result r{};
    r.n_clusters = hm[0];
    for (uint32_t k = 0; k < hm[0]; ++k) {
        r.largest = std::max(r.largest, hs[k]);
        if ((hf[k] & 3u) == 3u) r.spans |= 1u;
        if ((hf[k] & 12u) == 12u) r.spans |= 2u;
        if ((hf[k] & 48u) == 48u) r.spans |= 4u;
    }
    r.percolates = r.spans != 0;
    r.PL = N ? (double)r.largest / (double)N : 0.0;
    if (out) *out = r;
    if (sizes) {
        std::sort(hs.begin(), hs.end());
        std::copy(hs.begin(), hs.begin() + std::min<size_t>(hs.size(), sizes_cap), sizes);
    }
    return SCORE_OK;
}

}  // namespace score
