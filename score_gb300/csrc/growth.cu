// score_gb300 growth context: device memory layout, the per-step launch sequence
// and the host FP64 master-thread work (dt, physics, P on first use).
//
// HBM layout of one domain (N cells; list capacities cap_I = N, cap_B = N or the
// reference's 2(xy+xz+yz) Border limit):
//   grid   u32[N]   deformed id < ndefg | CURRENTLY_INFECTED | ndefg + rxg
//   claim  u32[N]   attempt ordinal of the first infection of this step (0xFFFFFFFF free)
//   front list L (SoA, slot-indexed): fill f64|f32, [comp f32], vel f64|f32, defg u32,
//          rxg u32, xyz u32, dir u8
//   full_L u32[cap_L], recyc_L u32[reccap_L]                 (rebuilt every step)
//   fmask_L, imask_L u32[cap_L/32], tcnt_L u32[2 cap_L/2048]  grow bit masks, tile counts
//   amask, tobm u32[N], ctcnt u32[2 N/256]                    per-full-cell attempt/win masks
//   ptab   u64[nrxg*ndefg] mobility weights P(rxg,defg), filled on first use
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/score_gb300.h"
#include "device_common.cuh"
#include "growth_kernels.cuh"
#include "host_model.h"
#include "percolation.h"

using namespace score;

namespace {

static_assert(offsetof(DevState, nfull) == kStepFieldsOffset, "per-step fields must start at kStepFieldsOffset");

// ------------------------------------------------------------------ small kernels
__global__ void k_count_defg(const uint32_t* grid, uint64_t n, uint32_t ndefg, uint32_t* cnt, uint32_t* err) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t g = grid[i];
        if (g < ndefg) atomicAdd(&cnt[g], 1u);
        else atomicOr(err, kErrBounds);
    }
}

__global__ void k_gather_u32(const uint32_t* src, const uint32_t* idx, uint32_t n, uint32_t* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = src[idx[i]];
}

struct NucRec { uint32_t list, slot, site, rxg, defg, pad; double P; };

// nucleus: fill 1.0 (ALMOST_FULLY_INFECTED), infector 26 (f_geo 1.0)
template <bool FP32>
__global__ void k_place_nuclei(DomainArgs a, const NucRec* rec, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const NucRec r = rec[i];
        const DFront& f = a.f[r.list];
        const double mo = mobility(a, r.P);
        const double v = velocity_from_mobility(a, mo, r.defg, 26);
        f.mob[r.slot] = mo;
        if (!FP32) { ((double*)f.fill)[r.slot] = 1.0; ((double*)f.vel)[r.slot] = v; }
        else { ((float*)f.fill)[r.slot] = 1.0f; f.comp[r.slot] = 0.0f; ((float*)f.vel)[r.slot] = (float)v; }
        f.dir[r.slot] = 26 | kStale;
        f.defg[r.slot] = r.defg;
        f.rxg[r.slot] = r.rxg;
        f.xyz[r.slot] = r.site;
        a.grid[r.site] = kCurrentlyInfected;
    }
}

// Nuclei due during the run, placed on the device so that the host needs no round trip:
// candidates in rxg order with the deformed grain of their site and P (computed by the
// host from the loaded grid: a site that is still deformed has its loaded grain).  A
// candidate is placed when its site is still deformed and no earlier candidate of the
// batch has the same site, exactly as the host placement decides; placed nuclei take
// the next slots of their list in candidate order.
struct NucDue { uint32_t site, rxg, defg, list; double P; };
constexpr uint32_t kDueMax = 1024;  // candidates per launch (one block)

template <bool FP32>
__global__ void __launch_bounds__(kDueMax) k_place_due(DomainArgs a, const NucDue* rec, uint32_t n) {
    __shared__ uint32_t s_site[kDueMax];
    __shared__ uint32_t s_wc[2][kDueMax / 32];
    __shared__ uint32_t s_base[2];
    const uint32_t i = threadIdx.x;
    const int warp = (int)(i >> 5), lane = (int)(i & 31);
    NucDue r{};
    if (i < n) { r = rec[i]; s_site[i] = r.site; }
    if (i == 0) { s_base[0] = a.st->next_never[0]; s_base[1] = a.st->next_never[1]; }
    __syncthreads();
    bool ok = false;
    if (i < n && r.site < a.ncells && r.list < 2) {
        ok = a.grid[r.site] < a.ndefg;
        for (uint32_t j = 0; j < i && ok; ++j) if (s_site[j] == r.site) ok = false;
    }
    const uint32_t b0 = __ballot_sync(0xFFFFFFFFu, ok && r.list == 0), b1 = __ballot_sync(0xFFFFFFFFu, ok && r.list == 1);
    if (lane == 0) { s_wc[0][warp] = __popc(b0); s_wc[1][warp] = __popc(b1); }
    __syncthreads();
    const int L = r.list == 1 ? 1 : 0;
    uint32_t rank = __popc((L ? b1 : b0) & lanemask_lt());
    for (int w = 0; w < warp; ++w) rank += s_wc[L][w];
    if (ok) {
        const uint32_t slot = s_base[L] + rank;
        const DFront& f = a.f[L];
        if (slot >= f.cap) {
            atomicOr(&a.st->err, kErrCapacity);
        } else if (L == 1 && a.border_policy == 0 && slot >= a.border_ref_cap) {
            atomicOr(&a.st->err, kErrBorderRef);
        } else {
            const double mo = mobility(a, r.P);
            const double v = velocity_from_mobility(a, mo, r.defg, 26);
            f.mob[slot] = mo;
            if (!FP32) { ((double*)f.fill)[slot] = 1.0; ((double*)f.vel)[slot] = v; }
            else { ((float*)f.fill)[slot] = 1.0f; f.comp[slot] = 0.0f; ((float*)f.vel)[slot] = (float)v; }
            f.dir[slot] = 26 | kStale;
            f.defg[slot] = r.defg;
            f.rxg[slot] = r.rxg;
            f.xyz[slot] = r.site;
            a.grid[r.site] = kCurrentlyInfected;
            a.ptab[(unsigned long long)r.rxg * a.ndefg + r.defg] = (unsigned long long)__double_as_longlong(r.P);
            if (r.P >= 0.0) atomicMax(&a.st->pmax_bits, (unsigned long long)__double_as_longlong(r.P));
        }
    }
    if (i == 0) {
        uint32_t t0 = 0, t1 = 0;
        for (int w = 0; w < (int)(kDueMax / 32); ++w) { t0 += s_wc[0][w]; t1 += s_wc[1][w]; }
        a.st->next_never[0] = s_base[0] + t0;
        a.st->next_never[1] = s_base[1] + t1;
        a.st->nnuc += t0 + t1;
    }
}

__global__ void k_clear_ptab(unsigned long long* ptab, const unsigned long long* idx, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) ptab[idx[i]] = kPtabEmpty;
}

__global__ void k_fill_ptab(unsigned long long* ptab, const unsigned long long* idx, const double* val, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        ptab[idx[i]] = (unsigned long long)__double_as_longlong(val[i]);
}

// new cells whose P arrived from the host: their velocity factor
template <bool FP32>
__global__ void k_labels_front(DomainArgs a, int L, uint32_t n, uint32_t* lab) {
    const DFront& f = a.f[L];
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        if (f.dir[s] == kInactive) continue;
        bool rx;
        if (!FP32) rx = !(((const double*)f.fill)[s] < 0.5);
        else rx = !((((const float*)f.fill)[s] - f.comp[s]) < 0.5f);
        int x, y, z;
        decode(a, f.xyz[s], x, y, z);
        lab[linear_of(a, x, y, z)] = rx ? a.ndefg + f.rxg[s] : f.defg[s];
    }
}

// the grid between the linear order of the C interface and the device's bricks (gindex); the
// padding words of odd extents hold kPadCell, which no attempt can claim
constexpr uint32_t kPadCell = 0xFFFFFFFFu;
__global__ void k_brick(DomainArgs a, const uint32_t* lin, uint32_t* g) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ncells; i += gridDim.x * blockDim.x) {
        int x, y, z;
        decode(a, i, x, y, z);
        g[i] = (x < (int)a.nx && y < (int)a.ny && z < (int)a.nz) ? lin[linear_of(a, x, y, z)] : kPadCell;
    }
}
__global__ void k_unbrick(DomainArgs a, const uint32_t* g, uint32_t* lin) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ncells; i += gridDim.x * blockDim.x) {
        int x, y, z;
        decode(a, i, x, y, z);
        if (x < (int)a.nx && y < (int)a.ny && z < (int)a.nz) lin[linear_of(a, x, y, z)] = g[i];
    }
}

// stable compaction of ACTIVE slots of list L into scratch arrays (ompshar_defragmentation,
// SCORE_Kernel.cpp:3877-3937), in three passes over tiles of kGrowTile slots like the
// grow step: count, one-block scan (k_scan_defrag), move.  Uses the list's tile counts.
__global__ void __launch_bounds__(kBlock) k_defrag_count(DomainArgs a, int L, uint32_t n) {
    const DFront fr = a.f[L];
    const uint32_t ntiles = (n + kGrowTile - 1) / kGrowTile;
    __shared__ uint32_t s_c[kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        uint32_t c = 0;
        for (int k = 0; k < kGrowItems; ++k) {
            const uint32_t s = tile * kGrowTile + (uint32_t)(k * kBlock) + threadIdx.x;
            c += __popc(__ballot_sync(0xFFFFFFFFu, s < n && fr.dir[s] != kInactive));
        }
        if (lane == 0) s_c[warp] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int w = 0; w < kWarps; ++w) t += s_c[w];
            fr.tcnt[2 * tile] = t;
            fr.tcnt[2 * tile + 1] = 0;
        }
        __syncthreads();
    }
}
__global__ void __launch_bounds__(1024) k_scan_defrag(DomainArgs a, int L, uint32_t n, uint32_t* out_count) {
    uint32_t tA, tB;
    scan_pairs_block(a.f[L].tcnt, (n + kGrowTile - 1) / kGrowTile, tA, tB);
    if (threadIdx.x == 0) *out_count = tA;
}
template <bool FP32>
__global__ void __launch_bounds__(kBlock) k_defrag_compact(DomainArgs a, int L, uint32_t n, DFront scratch) {
    constexpr int ITEMS = kGrowItems;
    const DFront fr = a.f[L];
    const uint32_t ntiles = (n + kGrowTile - 1) / kGrowTile;
    __shared__ uint32_t s_cntA[ITEMS * kWarps], s_cntB[ITEMS * kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t base = tile * kGrowTile;
        uint32_t am[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t s = base + (uint32_t)(k * kBlock) + threadIdx.x;
            am[k] = __ballot_sync(0xFFFFFFFFu, s < n && fr.dir[s] != kInactive);
            if (lane == 0) { s_cntA[k * kWarps + warp] = __popc(am[k]); s_cntB[k * kWarps + warp] = 0; }
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t tA, tB;
            scan64_pair(s_cntA, s_cntB, tA, tB);
        }
        __syncthreads();
        const uint32_t ex = fr.tcnt[2 * tile];
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (!((am[k] >> lane) & 1u)) continue;
            const uint32_t s = base + (uint32_t)(k * kBlock) + threadIdx.x;
            const uint32_t r = ex + s_cntA[k * kWarps + warp] + __popc(am[k] & lt);
            if (!FP32) {
                ((double*)scratch.fill)[r] = ((const double*)fr.fill)[s];
                ((double*)scratch.vel)[r] = ((const double*)fr.vel)[s];
                scratch.inc[r] = fr.inc[s];
                scratch.mob[r] = fr.mob[s];
            } else {
                ((float*)scratch.fill)[r] = ((const float*)fr.fill)[s];
                scratch.comp[r] = fr.comp[s];
                ((float*)scratch.vel)[r] = ((const float*)fr.vel)[s];
                scratch.mob[r] = fr.mob[s];
            }
            scratch.defg[r] = fr.defg[s]; scratch.rxg[r] = fr.rxg[s]; scratch.xyz[r] = fr.xyz[s]; scratch.dir[r] = fr.dir[s];
        }
        __syncthreads();
    }
}

// ---- on-the-fly characterization: RX area profile (log_rxareaprofile(threshold),
// SCORE_OnTheFlyCharacterization.cpp:274-384) over a label map, slices [z0, z1) ----
// section of every rx grain in every slice: hist[(z - z0) nrxg + rxg]; cells of one warp that
// carry the same label add together (a row of cells mostly belongs to one grain)
__global__ void k_area_hist(const uint32_t* lab, uint32_t nxy, uint32_t z0, uint32_t z1, uint32_t ndefg, uint32_t nrxg,
                            uint32_t* hist) {
    // cells and keys of a chunk fit 32 bits: N < 2^31 and the chunk's slices x nrxg <= N
    const uint64_t lo = (uint64_t)z0 * nxy;
    const uint32_t n = (z1 - z0) * nxy, stride = gridDim.x * blockDim.x;
    const uint32_t end = (n + 31u) & ~31u;  // whole warps, so that every lane takes part in the match
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < end; i += stride) {
        uint32_t key = 0xFFFFFFFFu;
        if (i < n) {
            const uint32_t r = lab[lo + i] - ndefg;  // wraps for deformed ids
            if (r < nrxg) key = (i / nxy) * nrxg + r;
        }
        const uint32_t m = __match_any_sync(0xFFFFFFFFu, key);
        if (key != 0xFFFFFFFFu && (__ffs(m) - 1) == (int)(threadIdx.x & 31)) atomicAdd(&hist[key], (uint32_t)__popc(m));
    }
}
// one block per slice: cells of the rx grains whose section reaches the threshold, and the rest;
// clears the slice's histogram for the next use
__global__ void __launch_bounds__(kBlock) k_area_sum(uint32_t* hist, uint32_t nrxg, uint32_t nxy, uint32_t thr, uint32_t* out) {
    __shared__ uint32_t s_w[kWarps];
    uint32_t* h = hist + (uint64_t)blockIdx.x * nrxg;
    uint32_t rx = 0;
    for (uint32_t r = threadIdx.x; r < nrxg; r += blockDim.x) {
        const uint32_t v = h[r];
        if (v >= thr) rx += v;
        h[r] = 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rx += __shfl_xor_sync(0xFFFFFFFFu, rx, o);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = rx;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kWarps; ++w) t += s_w[w];
        out[2 * blockIdx.x] = t;
        out[2 * blockIdx.x + 1] = nxy - t;
    }
}

// ---- ensemble post-processing (SCORE_SolitaryUnitAveraging.cpp) of the grain-evolution logs ----
struct EvoDev {
    const double* t;              // snapshot times
    const uint32_t* counts;       // nsnap x (ndefg + nrxg)
    const uint32_t* fin_defg;     // counts at the end of the run
    const uint32_t* fin_rxg;
    const uint32_t* cls;          // orientation class of every grain (macrotexture), or null
    uint32_t ndefg, nrxg, nsnap, pad;
    double tsimend, nboxvol;
};
// caHdl::get_interpCellCount (SCORE_SolitaryUnitAveraging.cpp:1304-1365) for grain `id`, with the
// snapshot index i of `when` (first snapshot at or after it) found once per time
__device__ __forceinline__ double interp_count(const EvoDev& e, uint32_t id, double when, uint32_t i) {
    const uint32_t G = e.ndefg + e.nrxg;
    if (when >= e.tsimend) return (double)(id < e.ndefg ? e.fin_defg[id] : e.fin_rxg[id - e.ndefg]);
    if (i > 0 && i < e.nsnap) {
        const double ti1 = e.t[i - 1], cnti1 = (double)e.counts[(uint64_t)(i - 1) * G + id];
        const double ti = e.t[i], cnti = (double)e.counts[(uint64_t)i * G + id];
        return __dadd_rn(cnti1, __dmul_rn(__dsub_rn(when, ti1), __ddiv_rn(__dsub_rn(cnti, cnti1), __dsub_rn(ti, ti1))));
    }
    if (i == 0) return (double)e.counts[id];
    return (double)e.counts[(uint64_t)(e.nsnap - 1) * G + id];
}
__device__ __forceinline__ uint32_t snap_index(const EvoDev& e, double when) {
    uint32_t i = 0;
    while (i < e.nsnap && e.t[i] < when) ++i;
    return i;
}
// one thread per (domain, time slot): the domain's interpolated deformed volume, summed over its
// grains in order (postprocess_rediscr_kinetics, :546-600), as box volume minus it
__global__ void k_rediscr_kinetics(const EvoDev* doms, uint32_t ndom, const double* when, uint32_t nslots, double* per_dom) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ndom * nslots) return;
    const uint32_t d = k / nslots, n = k - d * nslots;
    const EvoDev e = doms[d];
    const double w = when[n];
    const uint32_t i = snap_index(e, w);
    double dv = 0.0;
    for (uint32_t g = 0; g < e.ndefg; ++g) dv = __dadd_rn(dv, interp_count(e, g, w, i));
    per_dom[k] = __dsub_rn(e.nboxvol, dv);
}
// one thread per (domain, time slot): interpolated volume per orientation class, deformed grains then
// rx grains in order (postprocess_rediscr_macrotexture, :673-747); [domain][slot][class]
constexpr uint32_t kMaxClasses = 32;
__global__ void k_rediscr_texture(const EvoDev* doms, uint32_t ndom, const double* when, uint32_t nslots, uint32_t nclass,
                                  double* per_dom) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ndom * nslots) return;
    const uint32_t d = k / nslots, n = k - d * nslots;
    const EvoDev e = doms[d];
    const double w = when[n];
    const uint32_t i = snap_index(e, w);
    double acc[kMaxClasses];
    for (uint32_t c = 0; c < nclass; ++c) acc[c] = 0.0;
    for (uint32_t g = 0; g < e.ndefg + e.nrxg; ++g) {
        const uint32_t c = e.cls[g];
        acc[c] = __dadd_rn(acc[c], interp_count(e, g, w, i));
    }
    for (uint32_t c = 0; c < nclass; ++c) per_dom[(uint64_t)k * nclass + c] = acc[c];
}
// ensemble sums over the domains in order, one thread per output value
__global__ void k_rediscr_ensemble(const double* per_dom, uint32_t ndom, uint32_t m, double* out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double v = 0.0;
    for (uint32_t d = 0; d < ndom; ++d) v = __dadd_rn(v, per_dom[(uint64_t)d * m + k]);
    out[k] = v;
}

__global__ void k_first_inactive(const uint8_t* dir, uint32_t lo, uint32_t hi, uint32_t* out) {
    for (uint32_t s = lo + blockIdx.x * blockDim.x + threadIdx.x; s < hi; s += gridDim.x * blockDim.x)
        if (dir[s] == kInactive) atomicMin(out, s);
}

inline uint32_t blocks_for(uint64_t work, int sms, int per_sm = 8) {
    uint64_t b = (work + kBlock - 1) / kBlock;
    uint64_t cap = (uint64_t)sms * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (uint32_t)b;
}

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
}

}  // namespace

// ------------------------------------------------------------------ context
struct Engine;

struct score_ctx {
    score_params prm{};
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    std::string err;
    Physics ph;

    uint32_t nx = 0, ny = 0, nz = 0;
    uint64_t N = 0;
    uint64_t ncells = 0;               // grid words on the device (2x2x2 bricks over the extents rounded up to even)
    uint32_t ndefg = 0, nrxg = 0;
    bool loaded = false, fp32 = false, failed = false;
    int refresh = 0;                   // next step: 1 full refresh from P, 2 from cached mobilities
    std::vector<double> defg_q, rxg_q, rho0, rho, tincub;
    std::vector<uint32_t> site;        // nucleus sites, linear index (x + nx (y + ny z))
    std::vector<uint32_t> gsite;       // the same sites as grid words (brick index)
    std::vector<uint32_t> site_defg;   // deformed grain of each nucleus site in the loaded grid
    std::vector<uint8_t> placed;
    std::vector<uint32_t> nuc_order;   // rxg ids sorted by (tincub, id)
    size_t nuc_pos = 0;                // nuc_order[0, nuc_pos) already considered
    std::vector<uint32_t> defg_cnt_host, defg_cnt_init_host;
    std::vector<double> user_ptab;
    std::vector<double> pforce_host;
    double mob_host[4] = {0, 0, 0, 0};  // mobilities the front's vel factors were computed with
    double dt_cached = -1.0;             // dt the front's cached fill increments were computed with
    double pf_sig[2] = {0, 0};           // Gb^2/2 and drag the driving-force table was computed with
    uint64_t rho_version = 0, pf_rho_version = ~0ull, rhomax_version = ~0ull;
    std::vector<uint32_t> rho_order;   // deformed grains by descending rho0 (rho max while rho == rho0)
    size_t rho_cursor = 0;             // rho_order[0, cursor) have no cells left
    std::vector<double> rho_next;      // rho at the end of the running step (computed while it runs)
    bool ahead = false;                // physics_ahead ran for the running step

    DomainArgs a{};
    DevState* d_state = nullptr;
    DevState* h_state = nullptr;       // pinned host copy of the device scalars (load checks)
    HostBox* h_box = nullptr;          // pinned, device-mapped step mailbox
    HostBox* d_box = nullptr;          // its device address
    double* d_pforce = nullptr;
    double* h_pforce = nullptr;            // pinned staging of the driving forces
    NucDue* h_due = nullptr;               // pinned staging of nuclei due during the run
    NucDue* d_due = nullptr;
    uint32_t* d_grid_init = nullptr;       // the loaded deformed grid (restart source)
    uint32_t* d_defg_cnt_init = nullptr;   // its per-grain cell counts
    uint32_t* d_u32tmp = nullptr;
    void* d_stage = nullptr;
    size_t stage_cap = 0;
    DFront scratch{};
    uint32_t scratch_cap = 0;
    size_t scnt_words[2] = {0, 0}, csct_words = 0;  // supertile counter arrays (zeroed on reset)

    double Xcells = 0.0;
    uint32_t step = 0, defrag_cnt = 0, n_nuclei = 0;
    uint32_t next_never[2] = {0, 0}, high_water[2] = {0, 0};
    score_step_stats last{};

    Engine* eng = nullptr;             // launches this domain's steps (its own, or a batch's)
    bool own_eng = false;
    bool running = false;              // steps in the next batched step
    double weights_ms = 0.0;           // host time in requested weights (summed into the engine's timing)
    bool ans_ready = false;            // the engine computed this step's requested weights already
    std::vector<unsigned long long> ans_idx;  // weights computed for the last step's requests
    std::vector<double> ans_val;
    uint64_t launches = 0;             // kernels launched outside the step sequence
    std::vector<score_step_stats> trace;  // per-step stats of the last batched run
    // on-the-fly characterization: the grain-evolution log at the SingleGrainVolOverTime logpoints
    double t_step = 0.0;               // t at the start of the running step (the log records it)
    std::vector<double> log_cells;     // logpoint X times N: the reference's output_atthisX
    uint32_t log_next = 0;             // next logpoint
    std::vector<score_grainevo_info> log_info;
    uint32_t* d_log_counts = nullptr;  // log_cap x (ndefg + nrxg) cell counts
    uint32_t* d_log_area = nullptr;    // log_cap x 2 nz RX area profile
    uint32_t log_cap = 0;
    // P-table entries the runs since the last reset wrote (requests, nuclei): a reset clears these
    // instead of the whole table, unless the table is fresh or was loaded from the caller
    std::vector<unsigned long long> ptab_touched;
    bool ptab_dirty_all = true;

    ~score_ctx() { release_domain(); release_stream(); }
    void release_domain();
    void release_stream();
    int fail(int code, const std::string& msg) { err = msg; return code; }
    int cuda_fail(cudaError_t e, const char* what) {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return SCORE_ERR_CUDA;
    }
    bool stage(size_t bytes) {
        if (bytes <= stage_cap) return true;
        if (d_stage) cudaFree(d_stage);
        d_stage = nullptr; stage_cap = 0;
        if (cudaMalloc(&d_stage, bytes) != cudaSuccess) return false;
        stage_cap = bytes;
        return true;
    }
};

void score_ctx::release_domain() {
    if (device >= 0) cudaSetDevice(device);
    void* ptrs[] = {a.f[0].inc, a.f[1].inc, scratch.inc, a.f[0].mob, a.f[1].mob, scratch.mob, a.f[0].fill, a.f[0].comp, a.f[0].vel, a.f[0].defg, a.f[0].rxg, a.f[0].xyz, a.f[0].dir, a.f[0].full, a.f[0].recyc,
                    a.f[1].fill, a.f[1].comp, a.f[1].vel, a.f[1].defg, a.f[1].rxg, a.f[1].xyz, a.f[1].dir, a.f[1].full, a.f[1].recyc,
                    a.grid, a.claim, a.amask, a.ptab, a.defg_cnt, a.rxg_cnt, a.depleted, a.miss, a.tobm, a.ctcnt, a.fcell,
                    a.f[0].fmask, a.f[0].imask, a.f[0].tcnt, a.f[1].fmask, a.f[1].imask, a.f[1].tcnt,
                    a.f[0].scnt, a.f[1].scnt, a.csct,
                    d_state, d_pforce, d_u32tmp, d_stage, d_grid_init, d_defg_cnt_init, d_due, d_log_counts, d_log_area,
                    scratch.fill, scratch.comp, scratch.vel, scratch.defg, scratch.rxg, scratch.xyz, scratch.dir};
    for (void* p : ptrs) if (p) cudaFree(p);
    if (h_pforce) cudaFreeHost(h_pforce);
    h_pforce = nullptr;
    if (h_due) cudaFreeHost(h_due);
    h_due = nullptr; d_due = nullptr;
    a = DomainArgs{};
    scratch = DFront{};
    d_state = nullptr; d_pforce = nullptr; d_u32tmp = nullptr; d_stage = nullptr;
    d_grid_init = nullptr; d_defg_cnt_init = nullptr;
    d_log_counts = nullptr; d_log_area = nullptr; log_cap = 0;
    stage_cap = 0; scratch_cap = 0;
    loaded = false;
}


// ------------------------------------------------------------------ step engine
// Launches one growth step of every running domain of a set (one domain, or a batch of
// independent domains) as one sequence of kernels over all of them, on one stream:
// the per-domain argument blocks go to the device in one copy, the sequence runs as
// a CUDA graph (captured once per domain count and tile configuration) or as direct
// launches, and the step ends with one stream synchronization.
struct TuneCfg {
    int items = 8;          // grow tile = kBlock * items slots
    int fill_bpsm = 16;     // k_grow_fill blocks per SM
    int claim_bpsm = 2;     // k_claim blocks per SM (autotuner's choice on the 512^3 workload)
    int commit_bpsm = 8;    // k_resolve / k_commit blocks per SM (same)
    int spec_pct = 30;      // every slot's data loaded with its infector byte up to this INACTIVE share [%]
    int timing_every = 8;   // phase events on every k-th step of a run (0 never): each event costs
                            // microseconds of device time, so the steps in between run without
    bool operator==(const TuneCfg& o) const {
        return items == o.items && fill_bpsm == o.fill_bpsm && claim_bpsm == o.claim_bpsm && commit_bpsm == o.commit_bpsm;
    }
};

// Slots of the constant-memory argument array c_args, per device: each engine holds a
// contiguous range for as long as it lives.
std::mutex g_slot_mu;
uint64_t g_slots_used[64] = {};

int alloc_slots(int device, int n, int* base) {
    if (device < 0 || device >= 64 || n < 1 || n > kMaxDomains) return SCORE_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_slot_mu);
    for (int b = 0; b + n <= kMaxDomains; ++b) {
        const uint64_t m = (n == 64 ? ~0ull : ((1ull << n) - 1)) << b;
        if (!(g_slots_used[device] & m)) {
            g_slots_used[device] |= m;
            *base = b;
            return SCORE_OK;
        }
    }
    return SCORE_ERR_CAPACITY;
}

void free_slots(int device, int base, int n) {
    if (base < 0 || n < 1) return;
    std::lock_guard<std::mutex> lock(g_slot_mu);
    g_slots_used[device] &= ~((n == 64 ? ~0ull : ((1ull << n) - 1)) << base);
}

// Persistent worker threads for the per-domain host work of a batched step.
// Host worker threads for the per-domain and per-grain work between GPU steps.  A step's
// host work comes in short rounds a few hundred microseconds apart, so an idle worker spins
// (yielding) for up to kSpin before it sleeps: a round then starts and ends in about a
// microsecond instead of the tens of microseconds of a condition-variable wake-up.
// Jobs are handed out as tickets (round << 32 | index): a worker still finishing an older
// round can never take, or lose, a job of a newer one.
class WorkerPool {
public:
    explicit WorkerPool(unsigned n) {
        for (unsigned i = 0; i < n; ++i) th_.emplace_back([this] { loop(); });
    }
    ~WorkerPool() {
        {
            std::lock_guard<std::mutex> l(mu_);
            stop_.store(true);
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }
    // run f(0..n-1) on the workers and the calling thread; returns when all are done
    void run(int n, const std::function<void(int)>& f) {
        const uint64_t g = ++round_;
        ticket_.store(g << 32);  // first: tickets of the last round stop working
        job_.store(&f);
        njobs_.store((uint32_t)n);
        pending_.store(n);
        {
            std::lock_guard<std::mutex> l(mu_);
            gen_.store(g);
        }
        if (sleepers_.load() > 0) cv_.notify_all();
        work(g);
        while (pending_.load() > 0) std::this_thread::yield();
    }

private:
    static constexpr std::chrono::microseconds kSpin{2000};
    void work(uint64_t g) {
        for (;;) {
            uint64_t t = ticket_.load();
            for (;;) {
                if ((t >> 32) != g || (uint32_t)t >= njobs_.load()) return;
                if (ticket_.compare_exchange_weak(t, t + 1)) break;
            }
            (*job_.load())((int)(uint32_t)t);
            pending_.fetch_sub(1);
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            const auto t0 = std::chrono::steady_clock::now();
            while (gen_.load() == seen && !stop_.load()) {
                if (std::chrono::steady_clock::now() - t0 < kSpin) {
                    std::this_thread::yield();
                    continue;
                }
                std::unique_lock<std::mutex> l(mu_);
                sleepers_.fetch_add(1);
                cv_.wait(l, [&] { return stop_.load() || gen_.load() != seen; });
                sleepers_.fetch_sub(1);
            }
            if (stop_.load()) return;
            seen = gen_.load();
            work(seen);
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::atomic<const std::function<void(int)>*> job_{nullptr};
    std::atomic<uint64_t> ticket_{0}, gen_{0};
    std::atomic<uint32_t> njobs_{0};
    std::atomic<int> pending_{0}, sleepers_{0};
    std::atomic<bool> stop_{false};
    uint64_t round_ = 0;  // only the calling thread starts rounds
};

struct Engine {
    int device = 0, sms = 1;
    cudaStream_t stream = nullptr;
    bool fp32 = false;
    std::vector<score_ctx*> dom;
    int base = -1, nslots = 0;         // this engine's slots of c_args
    DomainArgs* d_args = nullptr;      // device address of c_args[base]
    DomainArgs* h_args = nullptr;      // pinned staging of the argument blocks
    std::vector<DomainArgs> h_args_dev;  // what the device's slots hold
    bool args_dirty = true;
    TuneCfg cfg;
    bool use_graph = true;
    bool capturing = false;
    bool events = false;               // the sequence being launched records the phase events
    int fill_mode = kFillAny;          // ... and the grow mode of every stepping domain (kFillAny: per domain)
    // the step without / with phase events, with the general / the refresh-only grow kernel
    // the step graphs: with or without phase events, times the fill mode (0..4, 5 for a batch of
    // cached increments, or per domain)
    static constexpr int kGraphs = 14;
    cudaGraphExec_t gexec[kGraphs] = {};
    TuneCfg gcfg[kGraphs];
    int gndom[kGraphs] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
    bool gfp32[kGraphs] = {};
    uint64_t run_steps = 0;            // steps since the run started (phase sampling)
    // 0 start, 1 end of fill, 2 end of lists, 3 end of claim, 4 end of step, 5/6 run span
    cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    score_timing tm{};
    uint64_t launches = 0;
    std::string err;
    std::unique_ptr<WorkerPool> pool;  // batches of several domains
    unsigned pool_threads = 0;         // workers of the pool (0: the caller's default)
    WorkerPool& workers(unsigned dflt) {
        if (!pool) pool.reset(new WorkerPool(std::max(1u, pool_threads ? pool_threads : std::min(dflt, std::thread::hardware_concurrency() - 1))));
        return *pool;
    }
    // the host's weights for all domains' requests, in pinned device-mapped memory: the
    // few cells that wait for them read them directly (no copy before the step)
    unsigned long long* h_ans_i = nullptr; double* h_ans_v = nullptr;
    unsigned long long* d_ans_i = nullptr; double* d_ans_v = nullptr;
    size_t ans_cap = 0, ans_total = 0;
    int stage_answers();

    ~Engine() { release(); }
    int init(int dev, int ndom) {
        device = dev;
        int s = alloc_slots(dev, ndom, &base);
        if (s != SCORE_OK) return s;
        nslots = ndom;
        cudaError_t e = cudaSetDevice(dev);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        for (auto& x : ev) if (e == cudaSuccess) e = cudaEventCreate(&x);
        void* sym = nullptr;
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&sym, c_args);
        if (e == cudaSuccess) d_args = (DomainArgs*)sym + base;
        if (e == cudaSuccess) e = cudaMallocHost((void**)&h_args, (size_t)ndom * sizeof(DomainArgs));
        h_args_dev.assign((size_t)ndom, DomainArgs{});
        args_dirty = true;
        return e == cudaSuccess ? SCORE_OK : SCORE_ERR_CUDA;
    }
    void drop_graph() {
        for (int k = 0; k < kGraphs; ++k) {
            if (gexec[k]) cudaGraphExecDestroy(gexec[k]);
            gexec[k] = nullptr;
            gndom[k] = -1;
        }
    }
    void release() {
        cudaSetDevice(device);
        drop_graph();
        if (h_ans_i) cudaFreeHost(h_ans_i);
        if (h_ans_v) cudaFreeHost(h_ans_v);
        h_ans_i = nullptr; h_ans_v = nullptr; d_ans_i = nullptr; d_ans_v = nullptr;
        ans_cap = ans_total = 0;
        if (h_args) cudaFreeHost(h_args);
        d_args = nullptr; h_args = nullptr;
        free_slots(device, base, nslots);
        base = -1; nslots = 0;
        for (auto& x : ev) if (x) { cudaEventDestroy(x); x = nullptr; }
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
    int fail(int code, const std::string& m) { err = m; return code; }
    void launch_sequence(int n);
    cudaError_t enqueue_step(int n, bool timed, int mode);
    int step(bool timed);
    void balance_weights();
    int run_until(double x_target, uint32_t max_steps, uint32_t* steps_done);
    int autotune(double x_target, uint32_t max_steps, score_tune* out);
    void get_tune(score_tune* out) const;
    int set_tune(const score_tune* t);
    void mark_run_start() { cudaEventRecord(ev[5], stream); run_steps = 0; }
    bool sample_step() const { return cfg.timing_every > 0 && run_steps % (uint64_t)cfg.timing_every == 0; }
    int mark_run_end();
};

namespace {
template <class Body>
void for_grains(score_ctx* c, Body body) {
    const size_t n = c->ndefg;
    Engine& E = *c->eng;
    if (n < 8192 || E.dom.size() != 1) { body(0, n); return; }
    E.workers(15);
    constexpr int kChunks = 16;
    E.pool->run(kChunks, [&](int k) { body(n * (size_t)k / kChunks, n * (size_t)(k + 1) / kChunks); });
}
}  // namespace

// (after Engine is complete: deleting it runs its destructor, which returns its
// argument slots, stream, events and pinned buffers)
void score_ctx::release_stream() {
    if (device >= 0) cudaSetDevice(device);
    if (h_state) cudaFreeHost(h_state);
    h_state = nullptr;
    if (h_box) cudaFreeHost(h_box);
    h_box = nullptr; d_box = nullptr;
    if (own_eng) delete eng;
    eng = nullptr;
    stream = nullptr;  // owned by the engine
}

// ------------------------------------------------------------------ helpers
namespace {

// Per-grain host loop over [0, ndefg): split over the engine's worker threads for a
// single domain with many grains (a batch already runs its domains in parallel).
template <class Body>
void for_grains(score_ctx* c, Body body);

// Driving force per deformed grain, the grow step's p (SCORE_Kernel.cpp:4082), from `rho`
// (whose version is `rho_ver`).  When it or the mobilities change, the front's velocity
// factors are recomputed in the next grow.  The copy is stream-ordered after every launch
// already enqueued, so a step in flight still reads the previous values.
int upload_physics(score_ctx* c, const double* rho, uint64_t rho_ver) {
    const double mob[4] = {c->ph.mLAGB, c->ph.mHAGB, c->ph.mGS, c->ph.mRHHAGB};
    const bool mob_same = memcmp(mob, c->mob_host, sizeof mob) == 0;
    // p depends on Gb^2/2, the drag and rho only: skip the per-grain pass when none changed
    const double sig[2] = {c->ph.Gbhalfsq, c->ph.zener()};
    if (mob_same && !c->pforce_host.empty() && memcmp(sig, c->pf_sig, sizeof sig) == 0 && c->pf_rho_version == rho_ver)
        return SCORE_OK;
    memcpy(c->pf_sig, sig, sizeof sig);
    c->pf_rho_version = rho_ver;
    // new p per grain, straight into the pinned staging buffer (its last copy to the device
    // finished before the step that just ended), noting whether any value changed
    if (c->pforce_host.size() != c->ndefg) c->pforce_host.assign(c->ndefg, std::numeric_limits<double>::quiet_NaN());
    std::atomic<bool> pf_changed{false};
    for_grains(c, [&](size_t lo, size_t hi) {
        bool ch = false;
        for (size_t g = lo; g < hi; ++g) {
            const double v = c->ph.driving_force(rho[g]);
            c->h_pforce[g] = v;
            if (v != c->pforce_host[g]) { c->pforce_host[g] = v; ch = true; }
        }
        if (ch) pf_changed.store(true);
    });
    if (!pf_changed.load() && mob_same) return SCORE_OK;
    c->refresh = (c->refresh == 1 || !mob_same) ? 1 : 2;  // new mobilities need P again
    memcpy(c->mob_host, mob, sizeof mob);
    if (!pf_changed.load()) return SCORE_OK;
    const cudaError_t e = cudaMemcpyAsync(c->d_pforce, c->h_pforce, (size_t)c->ndefg * 8, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "upload driving force");
    return SCORE_OK;
}

void set_step_args(score_ctx* c) {
    c->a.mLAGB = c->ph.mLAGB; c->a.mHAGB = c->ph.mHAGB; c->a.mGS = c->ph.mGS; c->a.mRH = c->ph.mRHHAGB;
    c->a.dt = c->ph.dt; c->a.cinv = (1.0 / c->prm.cellsize);
    c->a.dtc32 = (float)(c->ph.dt * (1.0 / c->prm.cellsize));
}

double weight_of(score_ctx* c, uint32_t r, uint32_t g) {
    if (!c->user_ptab.empty()) return c->user_ptab[(size_t)r * c->ndefg + g];
    return mobility_weight(c->prm, &c->rxg_q[4 * (size_t)r], &c->defg_q[4 * (size_t)g]);
}

// compute P for a list of table indices on the host, in parallel for large batches
void resolve_weights(score_ctx* c, const std::vector<unsigned long long>& idx, std::vector<double>& val) {
    val.resize(idx.size());
    auto work = [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i)  // a void slot (lost race) keeps 0, which no cell reads
            val[i] = idx[i] == kMissVoid ? 0.0 : weight_of(c, (uint32_t)(idx[i] / c->ndefg), (uint32_t)(idx[i] % c->ndefg));
    };
    size_t n = idx.size();
    Engine& E = *c->eng;
    if (n >= 16 && E.dom.size() == 1) {  // one domain: the engine's workers (a batch runs its domains in parallel)
        E.workers(15);
        const int chunks = (int)std::min<size_t>(64, n / 8);
        E.pool->run(chunks, [&](int k) { work(n * (size_t)k / chunks, n * (size_t)(k + 1) / chunks); });
        return;
    }
    // a batch computes its domains' weights on the engine's workers already: no nested threads
    unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096 || nth == 1 || E.dom.size() > 1) { work(0, n); return; }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t) th.emplace_back(work, n * t / nth, n * (t + 1) / nth);
    for (auto& t : th) t.join();
}

int check_device_errors(score_ctx* c, uint32_t flags) {
    if (!flags) return SCORE_OK;
    if (flags & kErrTimeout) return c->fail(SCORE_ERR_TIMEOUT, "a bounded device wait gave up (look-back scan)");
    if (flags & kErrKeyLimit) return c->fail(SCORE_ERR_KEYLIMIT, "more than 2^32-1 infection attempts in one step");
    if (flags & kErrBorderRef) return c->fail(SCORE_ERR_BORDER_CAPACITY, "Border list exceeded 2(xy+xz+yz) slots (the reference writes out of bounds here)");
    if (flags & kErrCapacity) return c->fail(SCORE_ERR_CAPACITY, "front list capacity exceeded");
    if (flags & kErrMissCap) return c->fail(SCORE_ERR_CAPACITY, "mobility-weight request list capacity exceeded");
    return c->fail(SCORE_ERR_STATE, "device bounds check failed (corrupt domain?)");
}

// site-saturated placement of nuclei with tincub <= t, rxg order
// (ompshar_sim_myCA_sitesaturatedNucleation / infect_JuvenileNucleation, SCORE_GrowthMachine.cpp:50-189)
// With `on_device`, up to kDueMax candidates are placed by k_place_due in stream order
// before the step (no host round trip); the placed count, the slots and the P max reach
// the host in the step's mailbox.  Otherwise the host reads the site values, decides and
// uploads the nuclei (two synchronizations).
int place_nuclei_upto(score_ctx* c, double tnow, uint32_t* nplaced, bool on_device) {
    std::vector<uint32_t> cand;
    while (c->nuc_pos < c->nuc_order.size() && c->tincub[c->nuc_order[c->nuc_pos]] <= tnow) cand.push_back(c->nuc_order[c->nuc_pos++]);
    std::sort(cand.begin(), cand.end());  // the reference places nuclei in rxg order
    if (nplaced) *nplaced = 0;
    if (cand.empty()) return SCORE_OK;
    const uint32_t n = (uint32_t)cand.size();
    if (on_device && n <= kDueMax) {
        const uint32_t nx = c->nx, ny = c->ny, nxy = nx * ny;
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t r = cand[i], s = c->site[r], g = c->site_defg[r];
            const uint32_t z = s / nxy, y = (s - z * nxy) / nx, x = s - z * nxy - y * nx;
            const bool inside = x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < c->nz - 1;
            c->placed[r] = 1;
            c->h_due[i] = NucDue{c->gsite[r], r, g, inside ? 0u : 1u, weight_of(c, r, g)};
            c->ptab_touched.push_back((unsigned long long)r * c->ndefg + g);
        }
        const cudaError_t e = cudaMemcpyAsync(c->d_due, c->h_due, (size_t)n * sizeof(NucDue), cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return c->cuda_fail(e, "upload due nuclei");
        set_step_args(c);
        if (c->fp32) k_place_due<true><<<1, kDueMax, 0, c->stream>>>(c->a, c->d_due, n);
        else k_place_due<false><<<1, kDueMax, 0, c->stream>>>(c->a, c->d_due, n);
        c->launches++;
        return SCORE_OK;
    }
    std::vector<uint32_t> sites(n), gsites(n), gval(n);
    for (uint32_t i = 0; i < n; ++i) { sites[i] = c->site[cand[i]]; gsites[i] = c->gsite[cand[i]]; }
    if (!c->stage((size_t)n * 8)) return c->fail(SCORE_ERR_NOMEM, "staging buffer");
    uint32_t* d_idx = (uint32_t*)c->d_stage;
    uint32_t* d_out = d_idx + n;
    cudaError_t e = cudaMemcpyAsync(d_idx, gsites.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "upload nucleus sites");
    k_gather_u32<<<blocks_for(n, c->sms), kBlock, 0, c->stream>>>(c->a.grid, d_idx, n, d_out);
    c->launches++;
    e = cudaMemcpyAsync(gval.data(), d_out, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "gather nucleus sites");

    std::vector<NucRec> recs;
    std::unordered_set<uint32_t> taken;
    std::vector<unsigned long long> pidx;
    std::vector<double> pval;
    const uint32_t nx = c->nx, ny = c->ny, nxy = nx * ny;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t r = cand[i];
        c->placed[r] = 1;
        uint32_t g = gval[i];
        if (taken.count(sites[i])) g = kCurrentlyInfected;
        if (g >= c->ndefg) continue;  // site already infected or recrystallized: nucleus not placeable
        const uint32_t s = sites[i];
        const uint32_t z = s / nxy, y = (s - z * nxy) / nx, x = s - z * nxy - y * nx;
        const bool inside = x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < c->nz - 1;
        const int L = inside ? 0 : 1;
        const uint32_t slot = c->next_never[L];
        if (slot >= c->a.f[L].cap) return c->fail(SCORE_ERR_CAPACITY, "front list capacity exceeded while placing nuclei");
        if (L == 1 && c->prm.border_policy == SCORE_BORDER_REFERENCE_LIMIT && slot >= c->a.border_ref_cap)
            return c->fail(SCORE_ERR_BORDER_CAPACITY, "Border list exceeded 2(xy+xz+yz) slots while placing nuclei");
        c->next_never[L]++;
        NucRec q{};
        q.list = (uint32_t)L; q.slot = slot; q.site = gsites[i]; q.rxg = r; q.defg = g;
        q.P = weight_of(c, r, g);
        if (q.P >= c->ph.Pmax) c->ph.Pmax = q.P;  // reg_myMobilityWeightMax, then the master's max
        recs.push_back(q);
        taken.insert(s);
        pidx.push_back((unsigned long long)r * c->ndefg + g);
        c->ptab_touched.push_back(pidx.back());
        pval.push_back(q.P);
        c->n_nuclei++;
        if (nplaced) (*nplaced)++;
    }
    if (recs.empty()) return SCORE_OK;
    const size_t nr = recs.size();
    const size_t bytes = nr * sizeof(NucRec) + nr * 16;
    if (!c->stage(bytes)) return c->fail(SCORE_ERR_NOMEM, "staging buffer");
    NucRec* d_rec = (NucRec*)c->d_stage;
    unsigned long long* d_pi = (unsigned long long*)(d_rec + nr);
    double* d_pv = (double*)(d_pi + nr);
    e = cudaMemcpyAsync(d_rec, recs.data(), nr * sizeof(NucRec), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_pi, pidx.data(), nr * 8, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_pv, pval.data(), nr * 8, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "upload nuclei");
    set_step_args(c);
    if (c->fp32) k_place_nuclei<true><<<blocks_for(nr, c->sms), kBlock, 0, c->stream>>>(c->a, d_rec, (uint32_t)nr);
    else k_place_nuclei<false><<<blocks_for(nr, c->sms), kBlock, 0, c->stream>>>(c->a, d_rec, (uint32_t)nr);
    k_fill_ptab<<<blocks_for(nr, c->sms), kBlock, 0, c->stream>>>(c->a.ptab, d_pi, d_pv, (uint32_t)nr);
    c->launches += 2;
    e = cudaMemcpyAsync((char*)c->d_state + offsetof(DevState, next_never), c->next_never, 8, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "place nuclei");
    for (int L = 0; L < 2; ++L) c->high_water[L] = std::max(c->high_water[L], c->next_never[L]);
    return SCORE_OK;
}

// ompshar_defragmentation, SCORE_Kernel.cpp:3877-3937, for one list
int defragment(score_ctx* c, int L) {
    const uint32_t n = c->next_never[L];
    if (n == 0) return SCORE_OK;
    DFront& fr = c->a.f[L];
    if (c->scratch_cap < n) {
        void* ptrs[] = {c->scratch.inc, c->scratch.mob, c->scratch.fill, c->scratch.comp, c->scratch.vel, c->scratch.defg, c->scratch.rxg, c->scratch.xyz, c->scratch.dir};
        for (void* p : ptrs) if (p) cudaFree(p);
        c->scratch = DFront{};
        const size_t fb = c->fp32 ? 4 : 8;
        cudaError_t e = cudaMalloc(&c->scratch.fill, (size_t)n * fb);
        if (e == cudaSuccess && c->fp32) e = cudaMalloc((void**)&c->scratch.comp, (size_t)n * 4);
        if (e == cudaSuccess) e = cudaMalloc(&c->scratch.vel, (size_t)n * fb);
        if (e == cudaSuccess && !c->fp32) e = dalloc(&c->scratch.inc, n);
        if (e == cudaSuccess) e = dalloc(&c->scratch.mob, n);
        if (e == cudaSuccess) e = dalloc(&c->scratch.defg, n);
        if (e == cudaSuccess) e = dalloc(&c->scratch.rxg, n);
        if (e == cudaSuccess) e = dalloc(&c->scratch.xyz, n);
        if (e == cudaSuccess) e = dalloc(&c->scratch.dir, n);
        if (e != cudaSuccess) return c->fail(SCORE_ERR_NOMEM, "defragmentation scratch");
        c->scratch_cap = n;
    }
    uint32_t* d_cnt = c->d_u32tmp;
    const uint32_t ntiles = (n + kGrowTile - 1) / kGrowTile;
    const uint32_t grid = std::min<uint32_t>(ntiles, (uint32_t)c->sms * 8);
    k_defrag_count<<<grid, kBlock, 0, c->stream>>>(c->a, L, n);
    k_scan_defrag<<<1, 1024, 0, c->stream>>>(c->a, L, n, d_cnt);
    if (c->fp32) k_defrag_compact<true><<<grid, kBlock, 0, c->stream>>>(c->a, L, n, c->scratch);
    else k_defrag_compact<false><<<grid, kBlock, 0, c->stream>>>(c->a, L, n, c->scratch);
    c->launches += 3;
    uint32_t active = 0;
    cudaError_t e = cudaMemcpyAsync(&active, d_cnt, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "defragment");
    if (active == n) {
        // no INACTIVE slot below next_never: the reference's scan for the first INACTIVE
        // continues into slots left behind by earlier compactions
        uint32_t first = c->high_water[L];
        if (c->high_water[L] > n) {
            e = cudaMemcpyAsync(d_cnt, &first, 4, cudaMemcpyHostToDevice, c->stream);
            k_first_inactive<<<blocks_for(c->high_water[L] - n, c->sms), kBlock, 0, c->stream>>>(fr.dir, n, c->high_water[L], d_cnt);
            c->launches++;
            if (e == cudaSuccess) e = cudaMemcpyAsync(&first, d_cnt, 4, cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess) return c->cuda_fail(e, "defragment");
        }
        c->next_never[L] = std::max(n, first);
    } else {
        const size_t fb = c->fp32 ? 4 : 8;
        e = cudaMemcpyAsync(fr.fill, c->scratch.fill, (size_t)active * fb, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess && c->fp32) e = cudaMemcpyAsync(fr.comp, c->scratch.comp, (size_t)active * 4, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fr.vel, c->scratch.vel, (size_t)active * fb, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess && !c->fp32) e = cudaMemcpyAsync(fr.inc, c->scratch.inc, (size_t)active * 8, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fr.mob, c->scratch.mob, (size_t)active * 8, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fr.defg, c->scratch.defg, (size_t)active * 4, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fr.rxg, c->scratch.rxg, (size_t)active * 4, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fr.xyz, c->scratch.xyz, (size_t)active * 4, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fr.dir, c->scratch.dir, (size_t)active, cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return c->cuda_fail(e, "defragment copy");
        c->next_never[L] = active;
    }
    e = cudaMemcpyAsync((char*)c->d_state + offsetof(DevState, next_never), c->next_never, 8, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "defragment");
    return SCORE_OK;
}

// Return the domain to its loaded state on the device (grid from the pristine copy,
// empty fronts, empty P cache) and redo the start of solve_RXGROWTH
// (SCORE_Kernel.cpp:6513-6530): rho max, T, G/b, mobilities, dt0.
int reset_state(score_ctx* c) {
    DomainArgs& a = c->a;
    const uint64_t W = c->ncells;
    cudaStream_t st = c->stream;
    cudaError_t e = cudaMemcpyAsync(a.grid, c->d_grid_init, W * 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.claim, 0xFF, W * 4, st);
    for (int L = 0; L < 2 && e == cudaSuccess; ++L) {
        e = cudaMemsetAsync(a.f[L].dir, kInactive, std::max<size_t>(c->high_water[L], 1), st);
    }
    if (e == cudaSuccess && c->user_ptab.empty()) {
        // every entry unknown again: the whole table after allocation or a caller's table, else only the
        // entries the last runs wrote (a 512^3 run writes about 0.03 % of its 8 GB table)
        const size_t total = std::max<size_t>((size_t)c->nrxg * c->ndefg, 1);
        const size_t nt = c->ptab_touched.size();
        if (c->failed) c->ptab_dirty_all = true;  // a step that failed may have tagged entries it never reported
        if (c->ptab_dirty_all || nt > total / 64 || !c->stage(nt * 8)) {
            e = cudaMemsetAsync(a.ptab, 0xFF, total * 8, st);
        } else if (nt) {
            e = cudaMemcpyAsync(c->d_stage, c->ptab_touched.data(), nt * 8, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) {
                k_clear_ptab<<<blocks_for(nt, c->sms), kBlock, 0, st>>>(a.ptab, (const unsigned long long*)c->d_stage, (uint32_t)nt);
                c->launches++;
                e = cudaGetLastError();
            }
        }
        c->ptab_touched.clear();
        c->ptab_dirty_all = false;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(a.defg_cnt, c->d_defg_cnt_init, (size_t)c->ndefg * 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.rxg_cnt, 0, std::max<size_t>(c->nrxg, 1) * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_state, 0, sizeof(DevState), st);
    for (int L = 0; L < 2 && e == cudaSuccess; ++L) e = cudaMemsetAsync(a.f[L].scnt, 0, c->scnt_words[L] * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.csct, 0, c->csct_words * 4, st);
    if (e != cudaSuccess) return c->cuda_fail(e, "reset domain");
    c->ans_idx.clear();
    c->ans_val.clear();
    c->log_info.clear();
    c->log_next = 0;
    c->log_cells.resize(std::min<uint32_t>(c->prm.n_logpoints, c->log_cap));
    for (size_t k = 0; k < c->log_cells.size(); ++k) c->log_cells[k] = c->prm.logpoint_x[k] * (double)c->N;  // log_initialization, :60-62
    memset(&c->h_box->snap, 0, sizeof(DevState));
    c->running = false;
    c->trace.clear();
    c->rho = c->rho0;
    c->defg_cnt_host = c->defg_cnt_init_host;
    c->placed.assign(c->nrxg, 0);
    c->nuc_pos = 0;
    Physics& ph = c->ph;
    ph.init(&c->prm);
    ph.rhomax = rhomax_of(c->rho, c->defg_cnt_host);
    c->rho_version = 0; c->rhomax_version = 0; c->pf_rho_version = ~0ull;
    c->rho_cursor = 0;
    ph.update_temperature();
    ph.update_atomistic();
    ph.update_mobilities();
    ph.dt = ph.dt_minimum();
    c->pforce_host.clear();
    memset(c->mob_host, 0, sizeof c->mob_host);
    c->ahead = false;
    int s = upload_physics(c, c->rho.data(), c->rho_version);
    if (s != SCORE_OK) return s;
    // the staging buffer is rewritten while the first step runs: its copy must be done
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return c->cuda_fail(e, "reset domain");
    c->refresh = 0;  // the front is empty; new cells get their factors when they are created
    c->dt_cached = -1.0;
    c->Xcells = 0.0; c->step = 0; c->defrag_cnt = 0; c->n_nuclei = 0;
    c->next_never[0] = c->next_never[1] = 0;
    c->high_water[0] = c->high_water[1] = 0;
    c->eng->tm = score_timing{};
    c->eng->mark_run_start();
    c->last = score_step_stats{};
    c->last.dt = ph.dt;
    c->last.rhomax = ph.rhomax;
    c->failed = false;
    c->loaded = true;
    return SCORE_OK;
}

}  // namespace

// ------------------------------------------------------------------ step of one domain, host side
namespace {

// Before the launch: time-dependent nucleation, defragmentation at X logpoints and the
// argument block of this step.
int pre_step(score_ctx* c, uint32_t* newnuc) {
    Physics& ph = c->ph;
    c->t_step = ph.t;
    // on-the-fly defragmentation at user X logpoints (SCORE_Kernel.cpp:6625-6630, thresholds in cells)
    const bool defrag = c->prm.defragmentation && c->defrag_cnt < c->prm.n_defrag && c->Xcells >= c->prm.defrag_x[c->defrag_cnt] * (double)c->N;
    // time-dependent nucleation (no-op when site-saturated); on the device unless the host
    // defragments this step (it needs the slot counts on the host)
    int s = place_nuclei_upto(c, ph.t, newnuc, !defrag);
    if (s != SCORE_OK) return s;
    if (defrag) {
        for (int L = 0; L < 2; ++L) { s = defragment(c, L); if (s != SCORE_OK) return s; }
        c->defrag_cnt++;
    }
    set_step_args(c);
    DomainArgs& a = c->a;
    a.dt_changed = (ph.dt != c->dt_cached) ? 1 : 0;
    a.refresh = c->refresh;
    // load strategy of k_grow_fill from the INACTIVE share of the last step's scanned slots
    const uint64_t scanned = (uint64_t)c->last.next_never[0] + c->last.next_never[1];
    a.spec = 100 * (scanned - std::min<uint64_t>(c->last.Sv, scanned)) <= (uint64_t)c->eng->cfg.spec_pct * scanned ? 1 : 0;
    a.active = 1;
    c->dt_cached = ph.dt;
    c->refresh = 0;
    return SCORE_OK;
}

bool recovering(const score_ctx* c) {
    return c->prm.recovery_model != SCORE_RECOVERY_NONE && c->prm.recovery_model != SCORE_RECOVERY_NES_SOLUTEDRAG;
}

// The part of the master block of solve_RXGROWTH (SCORE_Kernel.cpp:6691-6740) that does not
// depend on the step's outcome, run while the step is on the GPU: t + dt, temperature, G and
// b, drag, mobilities, the recovered rho (into rho_next: the rho max of the step still needs
// the current values) and the next step's driving forces.  The rest (P max, X, rho max, dt)
// follows in post_step, in the reference's order; none of it feeds back into this part.
int physics_ahead(score_ctx* c) {
    Physics& ph = c->ph;
    ph.t += ph.dt;
    ph.update_temperature();
    ph.update_atomistic();
    ph.update_microchemistry();
    ph.update_mobilities();
    c->ahead = true;
    if (!recovering(c)) return upload_physics(c, c->rho.data(), c->rho_version);
    c->rho_next.resize(c->ndefg);
    for_grains(c, [&](size_t lo, size_t hi) { ph.update_substructure(c->rho_next.data(), c->rho.data(), c->rho0.data(), lo, hi); });
    return upload_physics(c, c->rho_next.data(), c->rho_version + 1);
}

// log_OUTPUT_Diehl's grain-evolution branch (SCORE_OnTheFlyCharacterization.cpp:646-650), stream-ordered
// before the next step: every grain's cell count (log_grainevo, :478-531) and the RX area profile of
// the clarified labels (log_rxareaprofile(threshold), :274-384), on the device; the host keeps the
// snapshot's time (before t += dt), X, step and 32-bit Sv.
int log_snapshot(score_ctx* c, uint64_t Sv) {
    const uint32_t k = (uint32_t)c->log_info.size();
    if (k >= c->log_cap) return c->fail(SCORE_ERR_CAPACITY, "grain-evolution log full");
    cudaStream_t st = c->stream;
    DomainArgs& a = c->a;
    const size_t G = (size_t)c->ndefg + c->nrxg;
    uint32_t* cnt = c->d_log_counts + (size_t)k * G;
    cudaError_t e = cudaMemcpyAsync(cnt, a.defg_cnt, (size_t)c->ndefg * 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && c->nrxg) e = cudaMemcpyAsync(cnt + c->ndefg, a.rxg_cnt, (size_t)c->nrxg * 4, cudaMemcpyDeviceToDevice, st);
    // labels by the clarify rule into the attempt-mask array (free between steps)
    uint32_t* lab = a.amask;
    if (e == cudaSuccess) {
        k_unbrick<<<blocks_for(c->ncells, c->sms, 16), kBlock, 0, st>>>(a, a.grid, lab);
        c->launches++;
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return c->cuda_fail(e, "grain-evolution log");
    for (int L = 0; L < 2; ++L) {
        const uint32_t n = c->next_never[L];
        if (n == 0) continue;
        if (c->fp32) k_labels_front<true><<<blocks_for(n, c->sms), kBlock, 0, st>>>(a, L, n, lab);
        else k_labels_front<false><<<blocks_for(n, c->sms), kBlock, 0, st>>>(a, L, n, lab);
        c->launches++;
    }
    // per-slice sections of the rx grains, in chunks of slices whose histogram fits the win-mask array
    uint32_t* out = c->d_log_area + (size_t)k * 2 * c->nz;
    const uint32_t nxy = c->nx * c->ny, nr = std::max<uint32_t>(c->nrxg, 1);
    const uint32_t K = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(c->nz, c->N / nr));
    e = cudaMemsetAsync(a.tobm, 0, (size_t)K * nr * 4, st);
    if (e != cudaSuccess) return c->cuda_fail(e, "RX area profile");
    for (uint32_t z0 = 0; z0 < c->nz; z0 += K) {
        const uint32_t z1 = std::min(c->nz, z0 + K);
        k_area_hist<<<blocks_for((uint64_t)(z1 - z0) * nxy, c->sms, 16), kBlock, 0, st>>>(lab, nxy, z0, z1, c->ndefg, c->nrxg, a.tobm);
        k_area_sum<<<z1 - z0, kBlock, 0, st>>>(a.tobm, c->nrxg, nxy, c->prm.rxarea_threshold, out + 2 * (size_t)z0);
        c->launches += 2;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return c->cuda_fail(e, "RX area profile");
    score_grainevo_info info{};
    info.t = c->t_step;
    info.X = c->Xcells / (double)c->N;
    info.step = c->step;
    info.Sv = (uint32_t)Sv;
    c->log_info.push_back(info);
    return SCORE_OK;
}

// After the step: the mailbox (scalars, weight requests, depleted grains), the host's
// weights for the requests (applied at the start of the next step), and the rest of the
// master block of solve_RXGROWTH (SCORE_Kernel.cpp:6691-6740).
int post_step(score_ctx* c, uint32_t newnuc, score_step_stats* out) {
    Physics& ph = c->ph;
    DomainArgs& a = c->a;
    cudaStream_t st = c->stream;
    const DevState hs = c->h_box->snap;
    if (hs.err) { c->failed = true; return check_device_errors(c, hs.err); }
    const uint64_t Sv = hs.sv[0] + hs.sv[1], nfull = (uint64_t)hs.nfull[0] + hs.nfull[1], nnew = (uint64_t)hs.nwin[0] + hs.nwin[1];
    newnuc += hs.nnuc;  // nuclei the device placed before the grow
    c->n_nuclei += hs.nnuc;

    // mobility weights requested this step: computed on the host (FP64, libm)
    double pmax_new = 0.0;
    if (hs.pmax_bits) memcpy(&pmax_new, &hs.pmax_bits, 8);
    uint32_t nreq = 0;  // distinct weights requested (void race slots excluded)
    if (c->ans_ready) {  // computed by the engine over all domains' requests
        c->ans_ready = false;
        for (double v : c->ans_val) if (v > pmax_new) pmax_new = v;
        for (unsigned long long x : c->ans_idx) nreq += x != kMissVoid;
    } else if (hs.nmiss > 0) {
        c->ans_idx.clear();
        c->ans_val.clear();
        std::vector<unsigned long long> idx(hs.nmiss);
        std::vector<double> val;
        cudaError_t e = cudaSuccess;
        if (hs.nmiss <= kBoxMiss) {
            memcpy(idx.data(), c->h_box->miss, (size_t)hs.nmiss * 8);
        } else {
            e = cudaMemcpyAsync(idx.data(), a.miss, (size_t)hs.nmiss * 8, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return c->cuda_fail(e, "read misses");
        }
        const auto w_t0 = std::chrono::steady_clock::now();
        resolve_weights(c, idx, val);
        c->weights_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w_t0).count();
        for (double v : val) if (v > pmax_new) pmax_new = v;
        for (unsigned long long x : idx) nreq += x != kMissVoid;
        // staged by the engine into one host-to-device copy before the next step
        c->ans_idx.swap(idx);
        c->ans_val.swap(val);
    } else {
        c->ans_idx.clear();
        c->ans_val.clear();
    }
    for (unsigned long long x : c->ans_idx)
        if (x != kMissVoid) c->ptab_touched.push_back(x);
    // deformed grains that ran out of cells this step (synchronize_mydefpool_counts)
    if (hs.ndepleted > 0) {
        const uint32_t nd = std::min(hs.ndepleted, c->ndefg);
        if (nd <= kBoxDep) {
            for (uint32_t i = 0; i < nd; ++i) c->defg_cnt_host[c->h_box->depleted[i]] = 0;
        } else {
            std::vector<uint32_t> dep(nd);
            cudaError_t e = cudaMemcpyAsync(dep.data(), a.depleted, (size_t)nd * 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return c->cuda_fail(e, "read depleted grains");
            for (uint32_t g : dep) c->defg_cnt_host[g] = 0;
        }
        c->rhomax_version = ~0ull;  // the set of grains with cells left changed
    }
    for (int L = 0; L < 2; ++L) {
        c->next_never[L] = hs.next_never[L];
        c->high_water[L] = std::max(c->high_water[L], c->next_never[L]);
    }

    // master block, SCORE_Kernel.cpp:6691-6740
    const double dt_used = ph.dt;
    if (pmax_new >= ph.Pmax) ph.Pmax = pmax_new;  // running max over every P ever assigned, floored at 0
    c->Xcells = c->Xcells + (double)nfull;
    const double X = (c->Xcells / (double)c->N);
    if (c->rhomax_version != c->rho_version) {  // rho max only moves when rho or the grain set changes
        if (c->rho_version == 0 || c->prm.recovery_model == SCORE_RECOVERY_HYPERBOLIC) {
            // rho is rho0, or rho0 / (1 + k t) (same order): the first grain in descending-rho0
            // order that has cells
            while (c->rho_cursor < c->rho_order.size() && c->defg_cnt_host[c->rho_order[c->rho_cursor]] == 0) ++c->rho_cursor;
            const double best = c->rho_cursor < c->rho_order.size() ? c->rho[c->rho_order[c->rho_cursor]] : -1.0;
            ph.rhomax = (best >= kRhomaxWellAnnealed) ? best : kRhomaxWellAnnealed;
        } else {
            ph.rhomax = rhomax_of(c->rho, c->defg_cnt_host);
        }
        c->rhomax_version = c->rho_version;
    }
    const double rhomax_step = ph.rhomax;
    if (c->log_next < c->log_cells.size() && c->Xcells >= c->log_cells[c->log_next]) {
        const int ls = log_snapshot(c, Sv);
        if (ls != SCORE_OK) return ls;
        c->log_next++;
    }
    if (!c->ahead) {
        const int s = physics_ahead(c);
        if (s != SCORE_OK) return s;
    }
    c->ahead = false;
    if (recovering(c)) {
        c->rho.swap(c->rho_next);
        c->rho_version++;
    }
    ph.dt = ph.dt_minimum();
    c->step++;

    score_step_stats& o = c->last;
    o = score_step_stats{};
    o.step = c->step; o.n_nuclei = newnuc; o.t = ph.t; o.dt = ph.dt; o.dt_used = dt_used;
    o.Xcells = c->Xcells; o.X = X; o.Sv = Sv; o.n_full = nfull; o.n_new = nnew;
    o.Pmax = ph.Pmax; o.rhomax = rhomax_step; o.dXstep = 0.0;
    o.next_never[0] = c->next_never[0]; o.next_never[1] = c->next_never[1];
    o.n_recycled[0] = hs.nrec[0]; o.n_recycled[1] = hs.nrec[1];
    o.p_misses = nreq;
    if (out) *out = o;
    return SCORE_OK;
}

// the stop rule at the top of the step loop, SCORE_Kernel.cpp:6619
bool domain_done(const score_ctx* c, double xt) {
    const double X = c->Xcells / (double)c->N;
    return (c->Xcells >= (double)c->N) || (X > xt) || (c->step > c->prm.nmax) || (c->ph.t > c->ph.t_end) || (c->ph.t > c->prm.tmax);
}

// phase boundary: a real event record node when the sequence is captured into a graph
inline void record(const Engine& E, int k) {
    if (!E.events) return;
    if (E.capturing) cudaEventRecordWithFlags(E.ev[k], E.stream, cudaEventRecordExternal);
    else cudaEventRecord(E.ev[k], E.stream);
}

template <bool FP32, int ITEMS>
void launch_grow(const Engine& E, int n) {
    const uint32_t g = (uint32_t)(E.sms * E.cfg.fill_bpsm);
    const int m = E.fill_mode;  // a single domain's is one of 0..4
    if (n == 1) {
        if (m == 4 || (FP32 && m == 3)) {
            // FP32 keeps no increment (its fill step is vel dt / cellsize), so grow mode 3 is mode 0 there
            k_grow_fill_sparse<FP32, ITEMS><<<g, kBlock, 0, E.stream>>>(E.base);
        } else if (m == 1) {
            k_grow_fill<FP32, ITEMS, true, 1><<<g, kBlock, 0, E.stream>>>(E.base, n);
        } else if (m == 2) {
            k_grow_fill<FP32, ITEMS, true, 2><<<g, kBlock, 0, E.stream>>>(E.base, n);
        } else if constexpr (FP32) {
            k_grow_fill<true, ITEMS, true, 0><<<g, kBlock, 0, E.stream>>>(E.base, n);
        } else if (m == 0) {
            k_grow_fill_pf0<ITEMS><<<g, kBlock, 0, E.stream>>>(E.base);
        } else if constexpr (ITEMS <= 8) {
            k_grow_fill_pf<ITEMS><<<g, kBlock, 0, E.stream>>>(E.base);
        } else {
            k_grow_fill<false, ITEMS, true, 3><<<g, kBlock, 0, E.stream>>>(E.base, n);  // 16 items spill in the pipelined kernel
        }
    } else if (m == 5) {  // a batch whose domains all step from cached increments
        k_grow_fill_sparse_batch<FP32, ITEMS><<<g, kBlock, 0, E.stream>>>(E.base, n);
    } else if (m == 2) {
        k_grow_fill<FP32, ITEMS, false, 2><<<g, kBlock, 0, E.stream>>>(E.base, n);
    } else {
        k_grow_fill<FP32, ITEMS, false, kFillAny><<<g, kBlock, 0, E.stream>>>(E.base, n);
    }
    record(E, 1);
    k_grow_lists<ITEMS><<<(uint32_t)E.sms * 8, kBlock, 0, E.stream>>>(E.base, n);
}

template <bool FP32>
void launch_sequence_t(const Engine& E, int n) {
    cudaStream_t st = E.stream;
    const int d = E.base;
    const uint32_t S = (uint32_t)E.sms;
    record(E, 0);
    if (E.cfg.items == 4) launch_grow<FP32, 4>(E, n);
    else if (E.cfg.items == 16) launch_grow<FP32, 16>(E, n);
    else launch_grow<FP32, 8>(E, n);
    record(E, 2);
    if (n == 1) k_claim<true><<<S * (uint32_t)E.cfg.claim_bpsm, kBlock, 0, st>>>(d, n);
    else k_claim<false><<<S * (uint32_t)E.cfg.claim_bpsm, kBlock, 0, st>>>(d, n);
    record(E, 3);
    const uint32_t gt = (uint32_t)(kBlock * E.cfg.items);
    if (n == 1) {
        k_resolve<true><<<S * (uint32_t)E.cfg.commit_bpsm, kBlock, 0, st>>>(d, n);
        k_commit<FP32, true><<<S * (uint32_t)E.cfg.commit_bpsm, kBlock, 0, st>>>(d, n, gt);  // ends the step too
    } else {
        k_resolve<false><<<S * (uint32_t)E.cfg.commit_bpsm, kBlock, 0, st>>>(d, n);
        k_commit<FP32, false><<<S * (uint32_t)E.cfg.commit_bpsm, kBlock, 0, st>>>(d, n, gt);
        k_step_end<<<(uint32_t)n, kBlock, 0, st>>>(d, n, gt);
    }
    record(E, 4);
}

// kernels per step: fill, lists, claim, resolve, commit, and for batches a separate step end
inline int step_kernels(int n) { return n == 1 ? 5 : 6; }

}  // namespace

void Engine::launch_sequence(int n) {
    if (fp32) launch_sequence_t<true>(*this, n);
    else launch_sequence_t<false>(*this, n);
}

// the argument copy and the kernels of one step, as a graph replay or direct launches
cudaError_t Engine::enqueue_step(int n, bool timed, int mode) {
    // the argument blocks only change when dt, the physics or a domain's state changes
    cudaError_t e = cudaSuccess;
    if (args_dirty || memcmp(h_args, h_args_dev.data(), (size_t)n * sizeof(DomainArgs)) != 0) {
        e = cudaMemcpyAsync(d_args, h_args, (size_t)n * sizeof(DomainArgs), cudaMemcpyHostToDevice, stream);
        memcpy(h_args_dev.data(), h_args, (size_t)n * sizeof(DomainArgs));
        args_dirty = false;
    }
    if (e != cudaSuccess) return e;
    events = timed;
    fill_mode = mode;
    if (!use_graph) {
        launch_sequence(n);
        launches += step_kernels(n);
        return cudaGetLastError();
    }
    const int k = (timed ? 1 : 0) + 2 * (mode == kFillAny ? 6 : mode);
    if (!gexec[k] || gndom[k] != n || !(gcfg[k] == cfg) || gfp32[k] != fp32) {
        if (gexec[k]) cudaGraphExecDestroy(gexec[k]);
        gexec[k] = nullptr;
        gndom[k] = -1;
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        capturing = true;
        launch_sequence(n);
        capturing = false;
        e = cudaStreamEndCapture(stream, &g);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&gexec[k], g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) { gexec[k] = nullptr; return e; }
        gndom[k] = n; gcfg[k] = cfg; gfp32[k] = fp32;
    }
    launches += step_kernels(n);
    return cudaGraphLaunch(gexec[k], stream);
}

// Pack every domain's answered weights into the pinned, device-mapped staging buffer
// and point the domains' argument blocks at their part of it.
int Engine::stage_answers() {
    size_t total = 0;
    for (score_ctx* c : dom) total += c->ans_idx.size();
    ans_total = 0;
    if (total == 0) return SCORE_OK;
    if (total > ans_cap) {
        const size_t cap = std::max<size_t>(total, 2 * ans_cap);
        if (h_ans_i) cudaFreeHost(h_ans_i);
        if (h_ans_v) cudaFreeHost(h_ans_v);
        h_ans_i = nullptr; h_ans_v = nullptr; d_ans_i = nullptr; d_ans_v = nullptr;
        ans_cap = 0;
        cudaError_t e = cudaHostAlloc((void**)&h_ans_i, cap * 8, cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostAlloc((void**)&h_ans_v, cap * 8, cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&d_ans_i, h_ans_i, 0);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&d_ans_v, h_ans_v, 0);
        if (e != cudaSuccess) return fail(SCORE_ERR_NOMEM, "weight staging buffers");
        ans_cap = cap;
    }
    size_t off = 0;
    for (score_ctx* c : dom) {
        const size_t k = c->ans_idx.size();
        if (!k) continue;
        memcpy(h_ans_i + off, c->ans_idx.data(), k * 8);
        memcpy(h_ans_v + off, c->ans_val.data(), k * 8);
        c->a.ans_idx = d_ans_i + off;
        c->a.ans_val = d_ans_v + off;
        off += k;
    }
    ans_total = total;
    return SCORE_OK;
}

// The requested weights of all running domains of a batch, spread evenly over the workers:
// after nucleation a few domains request thousands of weights and would hold up a step
// whose post-processing gives each domain to one worker.  Few requests stay with their
// domain's post step.
void Engine::balance_weights() {
    std::vector<score_ctx*> req;
    std::vector<size_t> off(1, 0);
    for (score_ctx* c : dom) {
        c->ans_ready = false;
        if (!c->running) continue;
        const DevState& hs = c->h_box->snap;
        if (hs.err || hs.nmiss == 0 || hs.nmiss > kBoxMiss) continue;
        req.push_back(c);
        off.push_back(off.back() + hs.nmiss);
    }
    const size_t total = off.back();
    if (total < 512) return;
    const auto t0 = std::chrono::steady_clock::now();
    for (size_t j = 0; j < req.size(); ++j) {
        score_ctx* c = req[j];
        c->ans_idx.assign(c->h_box->miss, c->h_box->miss + (off[j + 1] - off[j]));
        c->ans_val.assign(off[j + 1] - off[j], 0.0);
        c->ans_ready = true;
    }
    constexpr size_t kChunk = 64;
    const int nchunks = (int)((total + kChunk - 1) / kChunk);
    workers(15);
    pool->run(nchunks, [&](int k) {
        const size_t lo = (size_t)k * kChunk, hi = std::min(total, lo + kChunk);
        size_t j = (size_t)(std::upper_bound(off.begin(), off.end(), lo) - off.begin()) - 1;
        for (size_t i = lo; i < hi; ++i) {
            while (i >= off[j + 1]) ++j;
            score_ctx* c = req[j];
            const unsigned long long x = c->ans_idx[i - off[j]];
            // a void slot (lost race) keeps 0, which no cell reads
            if (x != kMissVoid) c->ans_val[i - off[j]] = weight_of(c, (uint32_t)(x / c->ndefg), (uint32_t)(x % c->ndefg));
        }
    });
    tm.weights_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// One step of every running domain.
int Engine::step(bool timed) {
    cudaSetDevice(device);
    const auto host_t0 = std::chrono::steady_clock::now();
    const int n = (int)dom.size();
    std::vector<uint32_t> newnuc(n, 0);
    int nrun = 0;
    for (int i = 0; i < n; ++i) {
        score_ctx* c = dom[i];
        if (c->running) {
            const int s = pre_step(c, &newnuc[i]);
            if (s != SCORE_OK) return fail(s, c->err);
            ++nrun;
        } else {
            c->a.active = 0;
        }
        h_args[i] = c->a;
    }
    if (nrun == 0) return SCORE_OK;
    const auto pre_t1 = std::chrono::steady_clock::now();
    tm.pre_ms += std::chrono::duration<double, std::milli>(pre_t1 - host_t0).count();
    // the grow mode every stepping domain shares (a kernel specialised to it), or per domain
    int mode = -2;
    for (int i = 0; i < n; ++i) {
        if (!dom[i]->running) continue;
        const DomainArgs& a = h_args[i];
        // 0 cached increments, 1 / 2 refresh, 3 as 0 with few holes and dt unchanged, 4 as 0 with many holes
        const int m = a.refresh == 2 ? 2 : a.refresh == 1 ? 1 : !a.spec ? 4 : !a.dt_changed ? 3 : 0;
        mode = (mode == -2 || mode == m) ? m : kFillAny;
    }
    // batches: the gathered-slot kernel when no domain refreshes, the refresh-only kernel when all
    // refresh from cached mobilities, else the per-domain one
    if (n > 1 && mode != 2) {
        bool cached = true;
        for (int i = 0; i < n; ++i)
            if (dom[i]->running && h_args[i].refresh != 0) cached = false;
        mode = cached ? 5 : kFillAny;
    }
    cudaError_t e = enqueue_step(n, timed, mode);
    ++run_steps;
    // while the GPU steps: each domain's outcome-independent physics for the next step
    std::vector<int> status(n, SCORE_OK);
    if (e == cudaSuccess) {
        auto ahead = [&](int i) {
            score_ctx* c = dom[i];
            if (!c->running) return;
            cudaSetDevice(device);  // the calling thread may be a worker
            status[i] = physics_ahead(c);
        };
        if (n >= 4) {
            workers(15);
            pool->run(n, ahead);
        } else {
            for (int i = 0; i < n; ++i) ahead(i);
        }
    }
    const auto wait_t0 = std::chrono::steady_clock::now();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);  // the one wait of the step: the mailboxes are filled
    const auto wait_t1 = std::chrono::steady_clock::now();
    tm.wait_ms += std::chrono::duration<double, std::milli>(wait_t1 - wait_t0).count();
    if (e != cudaSuccess) {
        for (score_ctx* c : dom) c->failed = true;
        return fail(SCORE_ERR_CUDA, std::string("growth step: ") + cudaGetErrorString(e));
    }
    if (timed) {
        float f = 0, g = 0, cl = 0, cm = 0;
        e = cudaEventElapsedTime(&f, ev[0], ev[1]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&g, ev[0], ev[2]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&cl, ev[2], ev[3]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&cm, ev[3], ev[4]);
        if (e != cudaSuccess) return fail(SCORE_ERR_CUDA, std::string("phase timing: ") + cudaGetErrorString(e));
        tm.fill_ms += f; tm.grow_ms += g; tm.claim_ms += cl; tm.commit_ms += cm;
        tm.total_ms += g + cl + cm;
        tm.timed_steps += 1;
    }
    tm.grow_launches += 1;
    const double bpu = fp32 ? 21.0 : 25.0;  // algorithmic bytes per front-cell update of k_grow_fill
    for (int i = 0; i < n; ++i)
        if (status[i] != SCORE_OK) return fail(status[i], dom[i]->err);
    if (n >= 4) balance_weights();
    // the master-block work of each domain (weights, P max, X, rho max, dt) is independent
    auto post = [&](int i) {
        score_ctx* c = dom[i];
        if (!c->running) return;
        cudaSetDevice(device);  // the calling thread may be a worker
        status[i] = post_step(c, newnuc[i], nullptr);
    };
    if (n >= 4) {
        workers(15);
        pool->run(n, post);
    } else {
        for (int i = 0; i < n; ++i) post(i);
    }
    for (int i = 0; i < n; ++i) {
        score_ctx* c = dom[i];
        if (!c->running) continue;
        if (status[i] != SCORE_OK) return fail(status[i], c->err);
        const score_step_stats& st = c->last;
        if (timed) {  // bytes of the timed steps, so that bytes / time is a rate
            tm.grow_bytes += bpu * (double)st.Sv;
            tm.step_bytes += bpu * (double)st.Sv + 120.0 * (double)st.n_full + 37.0 * (double)st.n_new;
        }
        tm.weights_ms += c->weights_ms;
        c->weights_ms = 0.0;
    }
    const int sa = stage_answers();
    if (sa != SCORE_OK) return sa;
    tm.post_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wait_t1).count();
    tm.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host_t0).count();
    return SCORE_OK;
}

int Engine::mark_run_end() {
    cudaEventRecord(ev[6], stream);
    cudaError_t e = cudaEventSynchronize(ev[6]);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[5], ev[6]);
    if (e != cudaSuccess) return fail(SCORE_ERR_CUDA, std::string("run timing: ") + cudaGetErrorString(e));
    tm.run_ms = ms;
    return SCORE_OK;
}

// Step every domain until each meets its stop rule (X > x_target, time or step limits);
// a domain that stops leaves the launches, the others go on.  Each domain's per-step
// stats are kept in its trace.
int Engine::run_until(double x_target, uint32_t max_steps, uint32_t* steps_done) {
    uint32_t k = 0;
    for (;;) {
        int nrun = 0;
        for (score_ctx* c : dom) {
            const double xt = x_target < 0 ? c->prm.xmax : x_target;
            c->running = c->loaded && !c->failed && !domain_done(c, xt);
            nrun += c->running;
        }
        if (nrun == 0 || (max_steps && k >= max_steps)) break;
        const int s = step(sample_step());
        if (s != SCORE_OK) { if (steps_done) *steps_done = k; return s; }
        for (score_ctx* c : dom) if (c->running) c->trace.push_back(c->last);
        ++k;
    }
    for (score_ctx* c : dom) c->running = false;
    if (steps_done) *steps_done = k;
    return mark_run_end();
}

// ------------------------------------------------------------------ contexts
namespace {

int check_params(const score_params* p, int device) {
    if (p->nx < 3 || p->ny < 3 || p->nz < 3) return SCORE_ERR_ARG;
    const uint64_t N = (uint64_t)p->nx * p->ny * p->nz;
    if (N >= 0x7FFFFFFFull) return SCORE_ERR_ARG;  // slot counters and ranks are 32-bit with headroom
    if (8ull * ((p->nx + 1) / 2) * ((p->ny + 1) / 2) * ((p->nz + 1) / 2) >= 0x7FFFFFFFull) return SCORE_ERR_ARG;  // grid words
    if (p->n_schedule < 1) return SCORE_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return SCORE_ERR_NOT_BUILT; }
    if (device < 0 || device >= ndev) return SCORE_ERR_ARG;
    return SCORE_OK;
}

// a domain context stepped by `eng` (owned: a single-domain context; else a batch member)
int make_ctx(const score_params* p, Engine* eng, bool own, score_ctx** out) {
    score_ctx* c = new score_ctx();
    c->prm = *p;
    c->device = eng->device;
    c->nx = p->nx; c->ny = p->ny; c->nz = p->nz; c->N = (uint64_t)p->nx * p->ny * p->nz;
    c->ncells = 8ull * ((p->nx + 1) / 2) * ((p->ny + 1) / 2) * ((p->nz + 1) / 2);
    c->fp32 = p->precision == SCORE_PRECISION_FP32_KAHAN;
    c->eng = eng;
    c->own_eng = own;
    eng->dom.push_back(c);
    c->stream = eng->stream;
    c->sms = eng->sms;
    cudaError_t e = cudaMallocHost((void**)&c->h_state, sizeof(DevState));
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&c->h_box, sizeof(HostBox), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&c->d_box, c->h_box, 0);
    if (e != cudaSuccess) {
        eng->dom.pop_back();
        if (!own) c->eng = nullptr;
        delete c;
        return SCORE_ERR_CUDA;
    }
    memset(c->h_box, 0, sizeof(DevState));
    *out = c;
    return SCORE_OK;
}

}  // namespace

// ------------------------------------------------------------------ autotuner
// Runs real steps (results do not depend on the tile configuration: every compaction
// keeps slot order and claims are decided by ordinal) while cycling candidate
// configurations step by step, and keeps per kernel group the candidate with the least
// time per unit of work: k_grow_fill + k_grow_lists per front slot, k_claim per full
// cell, k_resolve + k_commit per full cell.  Direct launches while tuning.
int Engine::autotune(double x_target, uint32_t max_steps, score_tune* out) {
    static const int kItems[3] = {4, 8, 16};
    static const int kFill[4] = {4, 8, 16, 32};
    static const int kOther[4] = {2, 4, 8, 16};
    double ft[12] = {0}, fu[12] = {0}, ct[4] = {0}, cu[4] = {0}, mt[4] = {0}, mu[4] = {0};
    const bool graph = use_graph;
    use_graph = false;
    uint32_t k = 0;
    int status = SCORE_OK;
    for (;; ++k) {
        int nrun = 0;
        double slots = 0.0;
        for (score_ctx* c : dom) {
            const double xt = x_target < 0 ? c->prm.xmax : x_target;
            c->running = c->loaded && !c->failed && !domain_done(c, xt);
            if (c->running) { ++nrun; slots += (double)c->next_never[0] + (double)c->next_never[1]; }
        }
        if (nrun == 0 || (max_steps && k >= max_steps)) break;
        const int fi = (int)(k % 12), ci = (int)(k % 4), mi = (int)((k / 4) % 4);
        cfg.items = kItems[fi / 4];
        cfg.fill_bpsm = kFill[fi % 4];
        cfg.claim_bpsm = kOther[ci];
        cfg.commit_bpsm = kOther[mi];
        const score_timing before = tm;
        status = step(true);
        if (status != SCORE_OK) break;
        double full = 0.0;
        for (score_ctx* c : dom) if (c->running) full += (double)c->last.n_full;
        ft[fi] += tm.grow_ms - before.grow_ms; fu[fi] += slots;
        ct[ci] += tm.claim_ms - before.claim_ms; cu[ci] += full;
        mt[mi] += tm.commit_ms - before.commit_ms; mu[mi] += full;
    }
    for (score_ctx* c : dom) c->running = false;
    use_graph = graph;
    if (status != SCORE_OK) return status;
    auto best = [](const double* t, const double* u, int n) {
        int b = -1;
        for (int i = 0; i < n; ++i)
            if (u[i] > 0 && (b < 0 || t[i] / u[i] < t[b] / u[b])) b = i;
        return b;
    };
    const int bf = best(ft, fu, 12), bc = best(ct, cu, 4), bm = best(mt, mu, 4);
    TuneCfg t = cfg;  // the load strategy and the timing sample stay as they were set
    if (bf >= 0) { t.items = kItems[bf / 4]; t.fill_bpsm = kFill[bf % 4]; }
    if (bc >= 0) t.claim_bpsm = kOther[bc];
    if (bm >= 0) t.commit_bpsm = kOther[bm];
    cfg = t;
    if (out) {
        get_tune(out);
        out->fill_ns_per_slot = bf >= 0 ? 1e6 * ft[bf] / fu[bf] : 0.0;
        out->claim_ns_per_cell = bc >= 0 ? 1e6 * ct[bc] / cu[bc] : 0.0;
        out->commit_ns_per_cell = bm >= 0 ? 1e6 * mt[bm] / mu[bm] : 0.0;
        out->steps = k;
    }
    return SCORE_OK;
}

void Engine::get_tune(score_tune* out) const {
    *out = score_tune{};
    out->items = cfg.items;
    out->fill_blocks_per_sm = cfg.fill_bpsm;
    out->claim_blocks_per_sm = cfg.claim_bpsm;
    out->commit_blocks_per_sm = cfg.commit_bpsm;
    out->use_graph = use_graph ? 1 : 0;
    out->spec_holes_pct = cfg.spec_pct;
    out->timing_every = cfg.timing_every;
}

int Engine::set_tune(const score_tune* t) {
    if (t->items != 4 && t->items != 8 && t->items != 16) return fail(SCORE_ERR_ARG, "items must be 4, 8 or 16");
    for (int v : {t->fill_blocks_per_sm, t->claim_blocks_per_sm, t->commit_blocks_per_sm})
        if (v < 1 || v > 64) return fail(SCORE_ERR_ARG, "blocks per SM must be in 1..64");
    if (t->spec_holes_pct < 0 || t->spec_holes_pct > 100) return fail(SCORE_ERR_ARG, "spec_holes_pct must be in 0..100");
    if (t->timing_every < 0) return fail(SCORE_ERR_ARG, "timing_every must be >= 0");
    cfg.timing_every = t->timing_every;
    cfg.items = t->items;
    cfg.spec_pct = t->spec_holes_pct;
    cfg.fill_bpsm = t->fill_blocks_per_sm;
    cfg.claim_bpsm = t->claim_blocks_per_sm;
    cfg.commit_bpsm = t->commit_blocks_per_sm;
    use_graph = t->use_graph != 0;
    return SCORE_OK;
}

// ------------------------------------------------------------------ grain-evolution logs
namespace {

int grainevo_get(score_ctx* c, uint32_t i, score_grainevo_info* info, uint32_t* counts, uint32_t* rxarea) {
    if (i >= c->log_info.size()) return c->fail(SCORE_ERR_ARG, "no such grain-evolution snapshot");
    cudaSetDevice(c->device);
    if (info) *info = c->log_info[i];
    const size_t G = (size_t)c->ndefg + c->nrxg;
    cudaError_t e = cudaSuccess;
    if (counts) e = cudaMemcpyAsync(counts, c->d_log_counts + i * G, G * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && rxarea)
        e = cudaMemcpyAsync(rxarea, c->d_log_area + (size_t)i * 2 * c->nz, (size_t)2 * c->nz * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "read grain-evolution log");
    return SCORE_OK;
}

// Ensemble post-processing of the domains' grain-evolution logs on the device: kinetics (cls null)
// or macrotexture by orientation class.  Writes the time slots and [slot] or [slot][class] sums.
int rediscr(const std::vector<score_ctx*>& doms, uint32_t nslots, const uint32_t* cls, uint32_t nclass, double* t_out,
            double* out, double* boxvol_out, std::string& err) {
    if (doms.empty() || nslots < 2 || !t_out || !out) { err = "bad argument"; return SCORE_ERR_ARG; }
    if (cls && (nclass == 0 || nclass > kMaxClasses)) { err = "1 to 32 orientation classes"; return SCORE_ERR_ARG; }
    const int dev = doms[0]->device;
    double tmax = 0.0, box = 0.0;
    size_t ntimes = 0, ncls = 0;
    for (score_ctx* c : doms) {
        if (!c->loaded || c->device != dev) { err = "every domain must be loaded, on one device"; return SCORE_ERR_STATE; }
        // get_interpCellCount reads the first snapshot before the first log time: a domain needs one
        if (c->log_info.empty()) { err = "a domain has no grain-evolution snapshot (no logpoint reached)"; return SCORE_ERR_STATE; }
        if (c->ph.t >= tmax) tmax = c->ph.t;  // postprocess_init: the latest tsimend
        box = box + (double)c->N;
        ntimes += c->log_info.size();
        ncls += (size_t)c->ndefg + c->nrxg;
    }
    // postprocess_initrediscrtimes (REDISCR_TIME_EQUIDISTANT, tensmin 0)
    const double ttmin = 0.0, dt = (tmax - ttmin) / ((double)(nslots - 1));
    for (uint32_t n = 0; n < nslots; ++n) t_out[n] = ttmin + ((double)(n + 1) * dt);
    if (boxvol_out) *boxvol_out = box;
    cudaSetDevice(dev);
    for (score_ctx* c : doms) {  // every domain's last run is complete
        const cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { err = cudaGetErrorString(e); return SCORE_ERR_CUDA; }
    }
    const uint32_t ndom = (uint32_t)doms.size(), m = cls ? nslots * nclass : nslots;
    // one device block: domain descriptors, snapshot times, slot times, classes, per-domain and ensemble sums
    const size_t b_evo = ndom * sizeof(EvoDev), b_t = ntimes * 8, b_w = (size_t)nslots * 8, b_c = cls ? ncls * 4 : 0;
    const size_t b_pd = (size_t)ndom * m * 8, b_out = (size_t)m * 8;
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t total = up(b_evo) + up(b_t) + up(b_w) + up(b_c) + up(b_pd) + up(b_out);
    char* blk = nullptr;
    cudaError_t e = cudaMalloc((void**)&blk, total);
    if (e != cudaSuccess) { err = "post-processing buffers"; return SCORE_ERR_NOMEM; }
    EvoDev* d_evo = (EvoDev*)blk;
    double* d_t = (double*)(blk + up(b_evo));
    double* d_w = (double*)((char*)d_t + up(b_t));
    uint32_t* d_c = (uint32_t*)((char*)d_w + up(b_w));
    double* d_pd = (double*)((char*)d_c + up(b_c));
    double* d_out = (double*)((char*)d_pd + up(b_pd));
    std::vector<EvoDev> evo(ndom);
    std::vector<double> times;
    times.reserve(ntimes);
    size_t toff = 0, coff = 0;
    for (uint32_t d = 0; d < ndom; ++d) {
        score_ctx* c = doms[d];
        EvoDev& v = evo[d];
        v.t = d_t + toff;
        v.counts = c->d_log_counts;
        v.fin_defg = c->a.defg_cnt;
        v.fin_rxg = c->a.rxg_cnt;
        v.cls = cls ? d_c + coff : nullptr;
        v.ndefg = c->ndefg; v.nrxg = c->nrxg; v.nsnap = (uint32_t)c->log_info.size(); v.pad = 0;
        v.tsimend = c->ph.t; v.nboxvol = (double)c->N;
        for (const auto& info : c->log_info) times.push_back(info.t);
        toff += c->log_info.size();
        coff += (size_t)c->ndefg + c->nrxg;
    }
    cudaStream_t st = doms[0]->stream;
    e = cudaMemcpyAsync(d_evo, evo.data(), b_evo, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && b_t) e = cudaMemcpyAsync(d_t, times.data(), b_t, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, t_out, b_w, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && cls) e = cudaMemcpyAsync(d_c, cls, b_c, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const uint32_t nt = ndom * nslots;
        if (cls) k_rediscr_texture<<<(nt + 127) / 128, 128, 0, st>>>(d_evo, ndom, d_w, nslots, nclass, d_pd);
        else k_rediscr_kinetics<<<(nt + 127) / 128, 128, 0, st>>>(d_evo, ndom, d_w, nslots, d_pd);
        k_rediscr_ensemble<<<(m + 127) / 128, 128, 0, st>>>(d_pd, ndom, m, d_out);
        doms[0]->launches += 2;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, b_out, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(blk);
    if (e != cudaSuccess) { err = std::string("post-processing: ") + cudaGetErrorString(e); return SCORE_ERR_CUDA; }
    return SCORE_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

int score_abi_version(void) { return SCORE_ABI_VERSION; }

const char* score_status_string(int s) {
    switch (s) {
        case SCORE_OK: return "ok";
        case SCORE_ERR_ARG: return "bad argument";
        case SCORE_ERR_CUDA: return "CUDA error";
        case SCORE_ERR_NOMEM: return "out of memory";
        case SCORE_ERR_CAPACITY: return "front list capacity exceeded";
        case SCORE_ERR_BORDER_CAPACITY: return "Border list exceeded the reference's 2(xy+xz+yz) slots";
        case SCORE_ERR_TIMEOUT: return "bounded device wait gave up";
        case SCORE_ERR_STATE: return "call out of sequence";
        case SCORE_ERR_IO: return "input file error";
        case SCORE_ERR_KEYLIMIT: return "too many infection attempts in one step";
        case SCORE_ERR_NOT_BUILT: return "CUDA device unavailable";
        case SCORE_ERR_SCRATCH_LIMIT: return "input larger than the static scratch of a no-allocation entry point (nrxg > 65536)";
        default: return "unknown status";
    }
}

const char* score_last_error(const score_ctx* c) { return c ? c->err.c_str() : "null context"; }

int score_create(score_ctx** out, const score_params* p, int device) {
    if (!out || !p) return SCORE_ERR_ARG;
    *out = nullptr;
    int s = check_params(p, device);
    if (s != SCORE_OK) return s;
    Engine* eng = new Engine();
    s = eng->init(device, 1);
    if (s != SCORE_OK) { delete eng; return s; }
    eng->fp32 = p->precision == SCORE_PRECISION_FP32_KAHAN;
    score_ctx* c = nullptr;
    s = make_ctx(p, eng, true, &c);
    if (s != SCORE_OK) return s;
    *out = c;
    return SCORE_OK;
}

void score_destroy(score_ctx* c) { delete c; }

int score_load_domain(score_ctx* c, const uint32_t* grid, const double* defg_quat, const double* defg_rho0, uint32_t ndefg,
                      const double* rxg_quat, const uint32_t* rxg_site, const double* rxg_tincub, uint32_t nrxg,
                      const double* ptable) {
    if (!c || !grid || !defg_quat || !defg_rho0 || !rxg_quat || !rxg_site || ndefg == 0) return SCORE_ERR_ARG;
    if ((uint64_t)ndefg + nrxg >= 4096000000ull) return c->fail(SCORE_ERR_ARG, "too many grains");
    const uint64_t N = c->N;
    for (uint32_t r = 0; r < nrxg; ++r) if (rxg_site[r] >= N) return c->fail(SCORE_ERR_ARG, "nucleation site outside the domain");
    cudaSetDevice(c->device);
    // a context reloads in place when the pool sizes match; otherwise it reallocates
    const bool reuse = c->a.grid && c->ndefg == ndefg && c->nrxg == nrxg;
    if (!reuse && c->a.grid) c->release_domain();
    c->loaded = false;
    c->ndefg = ndefg; c->nrxg = nrxg;
    c->defg_q.assign(defg_quat, defg_quat + 4 * (size_t)ndefg);
    c->rxg_q.assign(rxg_quat, rxg_quat + 4 * (size_t)nrxg);
    c->rho0.assign(defg_rho0, defg_rho0 + ndefg);
    c->site.assign(rxg_site, rxg_site + nrxg);
    {
        const uint32_t gbx = (c->nx + 1) / 2, gby = (c->ny + 1) / 2, nxy = c->nx * c->ny;
        c->gsite.resize(nrxg);
        for (uint32_t r = 0; r < nrxg; ++r) {
            const uint32_t s = rxg_site[r], z = s / nxy, y = (s - z * nxy) / c->nx, x = s - z * nxy - y * c->nx;
            c->gsite[r] = gindex(gbx, gby, x, y, z);
        }
    }
    c->site_defg.resize(nrxg);
    for (uint32_t r = 0; r < nrxg; ++r) c->site_defg[r] = grid[rxg_site[r]];
    c->tincub.assign(nrxg, 0.0);
    if (rxg_tincub) c->tincub.assign(rxg_tincub, rxg_tincub + nrxg);
    c->rho_order.resize(ndefg);
    for (uint32_t g = 0; g < ndefg; ++g) c->rho_order[g] = g;
    std::stable_sort(c->rho_order.begin(), c->rho_order.end(), [&](uint32_t x, uint32_t y) { return c->rho0[x] > c->rho0[y]; });
    c->nuc_order.resize(nrxg);
    for (uint32_t r = 0; r < nrxg; ++r) c->nuc_order[r] = r;
    std::stable_sort(c->nuc_order.begin(), c->nuc_order.end(), [&](uint32_t x, uint32_t y) { return c->tincub[x] < c->tincub[y]; });
    c->user_ptab.clear();
    if (ptable) c->user_ptab.assign(ptable, ptable + (size_t)nrxg * ndefg);
    if (ptable || !reuse) c->ptab_dirty_all = true;  // a later reset without a caller's table clears it all

    const score_params& p = c->prm;
    DomainArgs& a = c->a;
    const size_t ptab_words = (size_t)nrxg * ndefg;
    cudaError_t e = cudaSuccess;
    if (!reuse) {
        a.nx = c->nx; a.ny = c->ny; a.nz = c->nz;
        a.gbx = (c->nx + 1) / 2; a.gby = (c->ny + 1) / 2; a.gbxy = a.gbx * a.gby;
        a.dgbx = make_fastdiv(a.gbx); a.dgbxy = make_fastdiv(a.gbxy);
        a.ncells = (uint32_t)c->ncells;
        a.ndefg = ndefg; a.nrxg = nrxg;
        a.border_ref_cap = 2 * ((c->nx * c->ny) + (c->nx * c->nz) + (c->ny * c->nz));
        a.border_policy = p.border_policy; a.boundary = p.boundary; a.mobility_model = p.mobility_model;
        // capacities: at most N infections ever happen, so N slots per list never overflow
        const uint32_t capI = (uint32_t)N;
        const uint32_t capB = (p.border_policy == SCORE_BORDER_REFERENCE_LIMIT) ? std::min<uint32_t>((uint32_t)N, a.border_ref_cap + 1) : (uint32_t)N;
        // recycle-list caps (ompshar_init_myRXFront{Inside,Border}, SCORE_Kernel.cpp:3615, 3670)
        const uint32_t recI = (uint32_t)(p.initial_cache * (double)N * p.maxfillperstep * kFullRecyclingFactor);
        const uint32_t recB = (uint32_t)((double)a.border_ref_cap * p.maxfillperstep * kFullRecyclingFactor);
        const uint32_t caps[2] = {capI, capB}, recs[2] = {recI, recB};
        const size_t fb = c->fp32 ? 4 : 8;
        for (int L = 0; L < 2; ++L) {
            DFront& f = a.f[L];
            f.cap = caps[L]; f.reccap = recs[L];
            if (e == cudaSuccess) e = cudaMalloc(&f.fill, (size_t)caps[L] * fb);
            if (e == cudaSuccess && c->fp32) e = cudaMalloc((void**)&f.comp, (size_t)caps[L] * 4);
            if (e == cudaSuccess) e = cudaMalloc(&f.vel, (size_t)caps[L] * fb);
            if (e == cudaSuccess && !c->fp32) e = dalloc(&f.inc, caps[L]);
            if (e == cudaSuccess) e = dalloc(&f.mob, caps[L]);
            if (e == cudaSuccess) e = dalloc(&f.defg, caps[L]);
            if (e == cudaSuccess) e = dalloc(&f.rxg, caps[L]);
            if (e == cudaSuccess) e = dalloc(&f.xyz, caps[L]);
            if (e == cudaSuccess) e = dalloc(&f.dir, caps[L]);
            if (e == cudaSuccess) e = dalloc(&f.full, caps[L]);
            if (e == cudaSuccess) e = dalloc(&f.recyc, recs[L]);
            // sized for the smallest grow tile (kBlock * 4 slots) and the largest (kBlock * 16)
            const size_t tiles = (size_t)caps[L] / (kBlock * 4) + 2;
            const size_t words = (size_t)caps[L] / 32 + 2 * GrowShape<16>::kWords;
            c->scnt_words[L] = 2 * (tiles / kSuper + 2);
            if (e == cudaSuccess) e = dalloc(&f.fmask, words);
            if (e == cudaSuccess) e = dalloc(&f.imask, words);
            if (e == cudaSuccess) e = dalloc(&f.tcnt, 2 * tiles * kWarps);
            if (e == cudaSuccess) e = dalloc(&f.scnt, c->scnt_words[L]);
        }
        c->csct_words = 2 * ((N / kBlock + 2) / kSuper + 2);
        a.misscap = (uint32_t)std::min<uint64_t>(N, 1ull << 25);
        if (e == cudaSuccess) e = dalloc(&a.grid, c->ncells);
        if (e == cudaSuccess) e = dalloc(&c->d_grid_init, c->ncells);
        if (e == cudaSuccess) e = dalloc(&a.claim, c->ncells);
        if (e == cudaSuccess) e = dalloc(&a.amask, N);
        if (e == cudaSuccess) e = dalloc(&a.tobm, N);
        if (e == cudaSuccess) e = dalloc(&a.fcell, N);
        if (e == cudaSuccess) e = dalloc(&a.ctcnt, 2 * (N / kBlock + 2));
        if (e == cudaSuccess) e = dalloc(&a.csct, c->csct_words);
        if (e == cudaSuccess) e = dalloc(&a.ptab, ptab_words);
        if (e == cudaSuccess) e = dalloc(&a.defg_cnt, ndefg);
        if (e == cudaSuccess) e = dalloc(&c->d_defg_cnt_init, ndefg);
        if (e == cudaSuccess) e = dalloc(&a.rxg_cnt, nrxg);
        if (e == cudaSuccess) e = dalloc(&a.depleted, ndefg);
        if (e == cudaSuccess) e = dalloc(&a.miss, a.misscap);
        if (e == cudaSuccess) e = dalloc(&c->d_state, 1);
        if (e == cudaSuccess) e = dalloc(&c->d_pforce, ndefg);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_pforce, std::max<size_t>(ndefg, 1) * 8);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_due, kDueMax * sizeof(NucDue));
        if (e == cudaSuccess) e = dalloc(&c->d_due, kDueMax);
        if (e == cudaSuccess) e = dalloc(&c->d_u32tmp, 64);
        // at most one grain-evolution snapshot per logpoint
        c->log_cap = std::min<uint32_t>(p.n_logpoints, SCORE_MAX_TABLE);
        if (e == cudaSuccess && c->log_cap) e = dalloc(&c->d_log_counts, (size_t)c->log_cap * (ndefg + nrxg));
        if (e == cudaSuccess && c->log_cap) e = dalloc(&c->d_log_area, (size_t)c->log_cap * 2 * c->nz);
        if (e != cudaSuccess) { c->release_domain(); return c->fail(SCORE_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(e)); }
        a.pforce = c->d_pforce;
        a.st = c->d_state;
        a.box = c->d_box;
        c->high_water[0] = a.f[0].cap; c->high_water[1] = a.f[1].cap;  // the reset clears every slot once
    } else {
        c->high_water[0] = std::max(c->high_water[0], c->next_never[0]);
        c->high_water[1] = std::max(c->high_water[1], c->next_never[1]);
    }
    // the linear grid goes through the claim array (reset before the first step) into bricks
    e = cudaMemcpyAsync(a.claim, grid, N * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && ptable) e = cudaMemcpyAsync(a.ptab, ptable, ptab_words * 8, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_defg_cnt_init, 0, (size_t)ndefg * 4, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_state, 0, sizeof(DevState), c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "load domain");
    // per-grain cell counts (solve_REPLACE_CA_STRUCTURE, SCORE_Kernel.cpp:6394-6400)
    k_count_defg<<<blocks_for(N, c->sms, 16), kBlock, 0, c->stream>>>(a.claim, N, ndefg, c->d_defg_cnt_init,
                                                                      (uint32_t*)((char*)c->d_state + offsetof(DevState, err)));
    k_brick<<<blocks_for(c->ncells, c->sms, 16), kBlock, 0, c->stream>>>(a, a.claim, c->d_grid_init);
    c->launches += 2;
    c->defg_cnt_init_host.assign(ndefg, 0);
    e = cudaMemcpyAsync(c->defg_cnt_init_host.data(), c->d_defg_cnt_init, (size_t)ndefg * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_state, c->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "count grains");
    if (c->h_state->err) return c->fail(SCORE_ERR_ARG, "grid holds ids >= ndefg");
    return reset_state(c);
}

int score_restart(score_ctx* c) {
    if (!c) return SCORE_ERR_ARG;
    if (!c->a.grid || c->ndefg == 0) return c->fail(SCORE_ERR_STATE, "no domain loaded");
    cudaSetDevice(c->device);
    c->high_water[0] = std::max(c->high_water[0], c->next_never[0]);
    c->high_water[1] = std::max(c->high_water[1], c->next_never[1]);
    return reset_state(c);
}

int score_place_nuclei(score_ctx* c, uint32_t* n_placed) {
    if (!c) return SCORE_ERR_ARG;
    if (!c->loaded) return c->fail(SCORE_ERR_STATE, "no domain loaded");
    if (c->failed) return SCORE_ERR_STATE;
    cudaSetDevice(c->device);
    return place_nuclei_upto(c, c->ph.t, n_placed, false);
}

int score_step(score_ctx* c, score_step_stats* out) {
    if (!c) return SCORE_ERR_ARG;
    if (!c->loaded) return c->fail(SCORE_ERR_STATE, "no domain loaded");
    if (c->failed) return SCORE_ERR_STATE;  // a device error left the front lists undefined
    c->running = true;
    const int s = c->eng->step(c->eng->sample_step());
    c->running = false;
    if (s != SCORE_OK) { if (c->err.empty()) c->err = c->eng->err; return s; }
    if (out) *out = c->last;
    return SCORE_OK;
}

int score_run_until(score_ctx* c, double x_target, score_step_stats* trace, uint32_t trace_cap, uint32_t* n_steps) {
    if (!c) return SCORE_ERR_ARG;
    if (!c->loaded) return c->fail(SCORE_ERR_STATE, "no domain loaded");
    if (c->failed) return SCORE_ERR_STATE;
    c->trace.clear();
    uint32_t k = 0;
    const int s = c->eng->run_until(x_target, 0, &k);
    if (trace) for (uint32_t i = 0; i < k && i < trace_cap && i < c->trace.size(); ++i) trace[i] = c->trace[i];
    if (n_steps) *n_steps = k;
    if (s != SCORE_OK && c->err.empty()) c->err = c->eng->err;
    return s;
}

int score_get_stats(score_ctx* c, score_step_stats* out) {
    if (!c || !out) return SCORE_ERR_ARG;
    *out = c->last;
    out->step = c->step; out->t = c->ph.t; out->dt = c->ph.dt; out->Xcells = c->Xcells;
    out->X = c->N ? c->Xcells / (double)c->N : 0.0; out->Pmax = c->ph.Pmax;
    return SCORE_OK;
}

int score_export_labels(score_ctx* c, uint32_t* labels) {
    if (!c || !labels) return SCORE_ERR_ARG;
    if (!c->loaded) return c->fail(SCORE_ERR_STATE, "no domain loaded");
    cudaSetDevice(c->device);
    uint32_t* d_lab = c->a.amask;  // N words, free between steps
    k_unbrick<<<blocks_for(c->ncells, c->sms, 16), kBlock, 0, c->stream>>>(c->a, c->a.grid, d_lab);
    c->launches++;
    cudaError_t e = cudaGetLastError();
    for (int L = 0; L < 2 && e == cudaSuccess; ++L) {
        const uint32_t n = c->next_never[L];
        if (n == 0) continue;
        if (c->fp32) k_labels_front<true><<<blocks_for(n, c->sms), kBlock, 0, c->stream>>>(c->a, L, n, d_lab);
        else k_labels_front<false><<<blocks_for(n, c->sms), kBlock, 0, c->stream>>>(c->a, L, n, d_lab);
        c->launches++;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(labels, d_lab, c->N * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "export labels");
    return SCORE_OK;
}

int score_grain_counts(score_ctx* c, uint32_t* rxg_counts, uint32_t* defg_counts) {
    if (!c) return SCORE_ERR_ARG;
    if (!c->loaded) return c->fail(SCORE_ERR_STATE, "no domain loaded");
    cudaSetDevice(c->device);
    cudaError_t e = cudaSuccess;
    if (rxg_counts && c->nrxg) e = cudaMemcpyAsync(rxg_counts, c->a.rxg_cnt, (size_t)c->nrxg * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && defg_counts) e = cudaMemcpyAsync(defg_counts, c->a.defg_cnt, (size_t)c->ndefg * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "grain counts");
    return SCORE_OK;
}

int score_grainevo_count(score_ctx* c, uint32_t* n) {
    if (!c || !n) return SCORE_ERR_ARG;
    *n = (uint32_t)c->log_info.size();
    return SCORE_OK;
}

int score_grainevo(score_ctx* c, uint32_t i, score_grainevo_info* info, uint32_t* counts, uint32_t* rxarea) {
    if (!c) return SCORE_ERR_ARG;
    return grainevo_get(c, i, info, counts, rxarea);
}

int score_rediscr_kinetics(score_ctx* c, uint32_t nslots, double* t_out, double* rxvol_out, double* boxvol_out) {
    if (!c) return SCORE_ERR_ARG;
    const int s = rediscr({c}, nslots, nullptr, 0, t_out, rxvol_out, boxvol_out, c->err);
    return s;
}

int score_percolation_analyze(score_ctx* c, int mode, score_perc_result* out, uint32_t* sizes, uint32_t sizes_cap, uint32_t* labels) {
    if (!c) return SCORE_ERR_ARG;
    if (!c->loaded) return c->fail(SCORE_ERR_STATE, "no domain loaded");
    cudaSetDevice(c->device);
    // the analysis reads the grid in linear order: a copy in the attempt-mask array (free between steps)
    k_unbrick<<<blocks_for(c->ncells, c->sms, 16), kBlock, 0, c->stream>>>(c->a, c->a.grid, c->a.amask);
    c->launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c->cuda_fail(e, "percolation grid");
    return percolation_analyze(c->a.amask, c->nx, c->ny, c->nz, c->ndefg, mode, c->stream, c->sms, out, sizes, sizes_cap, labels, c->err);
}

int score_get_timing(score_ctx* c, score_timing* out) {
    if (!c || !out) return SCORE_ERR_ARG;
    *out = c->eng->tm;
    out->kernel_launches = c->launches + c->eng->launches;
    return SCORE_OK;
}

int score_get_tune(score_ctx* c, score_tune* out) {
    if (!c || !out) return SCORE_ERR_ARG;
    c->eng->get_tune(out);
    return SCORE_OK;
}

int score_set_tune(score_ctx* c, const score_tune* t) {
    if (!c || !t) return SCORE_ERR_ARG;
    const int s = c->eng->set_tune(t);
    if (s != SCORE_OK) c->err = c->eng->err;
    return s;
}

int score_autotune(score_ctx* c, double x_target, uint32_t max_steps, score_tune* out) {
    if (!c) return SCORE_ERR_ARG;
    int s = score_restart(c);
    if (s == SCORE_OK) s = score_place_nuclei(c, nullptr);
    if (s == SCORE_OK) s = c->eng->autotune(x_target, max_steps, out);
    if (s != SCORE_OK) { if (c->err.empty()) c->err = c->eng->err; return s; }
    s = score_restart(c);
    if (s == SCORE_OK) s = score_place_nuclei(c, nullptr);
    return s;
}

}  // extern "C"

// ------------------------------------------------------------------ batched ensemble
// A batch splits its domains into groups of about equal cell count, each stepped by its own
// engine (stream, argument slots, graphs, workers) from its own host thread: the groups'
// latency-bound kernels overlap on the GPU and their host work overlaps on the CPU.  Within a
// group the domains step in lock-step, one sequence of launches per step.
struct score_batch {
    std::vector<std::unique_ptr<Engine>> engs;
    std::vector<score_ctx*> dom;
    std::string err;
    ~score_batch() {
        for (score_ctx* c : dom) delete c;
        dom.clear();
    }
    int fail(int code, const std::string& m) { err = m; return code; }
    int dom_fail(score_ctx* c, int code) { err = c->err; return code; }
    // f(g) for every group on its own thread (the calling thread takes group 0); first error wins
    template <class F>
    int each_group(F f) {
        const size_t G = engs.size();
        std::vector<int> st(G, SCORE_OK);
        std::vector<std::thread> th;
        for (size_t g = 1; g < G; ++g) th.emplace_back([&, g] { st[g] = f(g); });
        st[0] = f(0);
        for (auto& t : th) t.join();
        for (size_t g = 0; g < G; ++g)
            if (st[g] != SCORE_OK) return fail(st[g], engs[g]->err);
        return SCORE_OK;
    }
};

namespace {
constexpr uint32_t kGroupDomains = 32;  // domains per group (per engine and stream) of a batch
}

extern "C" {

int score_batch_create(score_batch** out, const score_params* params, uint32_t n, int device) {
    if (!out || !params || n == 0 || n > (uint32_t)kMaxDomains) return SCORE_ERR_ARG;
    *out = nullptr;
    for (uint32_t i = 0; i < n; ++i) {
        const int s = check_params(&params[i], device);
        if (s != SCORE_OK) return s;
        if (params[i].precision != params[0].precision) return SCORE_ERR_ARG;  // one precision per batch
    }
    score_batch* b = new score_batch();
    // groups of about equal cell count: largest domain first, to the lightest group
    const uint32_t G = std::max(1u, std::min(n / kGroupDomains, 4u));
    std::vector<uint32_t> order(n), group(n), count(G, 0);
    std::vector<uint64_t> load(G, 0);
    for (uint32_t i = 0; i < n; ++i) order[i] = i;
    auto cells = [&](uint32_t i) { return (uint64_t)params[i].nx * params[i].ny * params[i].nz; };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return cells(x) > cells(y); });
    for (uint32_t i : order) {
        const uint32_t g = (uint32_t)(std::min_element(load.begin(), load.end()) - load.begin());
        group[i] = g; load[g] += cells(i); ++count[g];
    }
    const unsigned hw = std::max(2u, std::thread::hardware_concurrency());
    for (uint32_t g = 0; g < G; ++g) {
        b->engs.emplace_back(new Engine());
        Engine& E = *b->engs.back();
        const int si = E.init(device, (int)count[g]);
        if (si != SCORE_OK) { delete b; return si; }
        E.fp32 = params[0].precision == SCORE_PRECISION_FP32_KAHAN;
        E.pool_threads = std::max(1u, (hw - 1) / G);
    }
    for (uint32_t i = 0; i < n; ++i) {
        score_ctx* c = nullptr;
        const int s = make_ctx(&params[i], b->engs[group[i]].get(), false, &c);
        if (s != SCORE_OK) { delete b; return s; }
        b->dom.push_back(c);
    }
    *out = b;
    return SCORE_OK;
}

void score_batch_destroy(score_batch* b) { delete b; }

const char* score_batch_last_error(const score_batch* b) { return b ? b->err.c_str() : "null batch"; }

int score_batch_load_domain(score_batch* b, uint32_t d, const uint32_t* grid, const double* defg_quat,
                            const double* defg_rho0, uint32_t ndefg, const double* rxg_quat, const uint32_t* rxg_site,
                            const double* rxg_tincub, uint32_t nrxg, const double* ptable) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    const int s = score_load_domain(b->dom[d], grid, defg_quat, defg_rho0, ndefg, rxg_quat, rxg_site, rxg_tincub, nrxg, ptable);
    return s == SCORE_OK ? s : b->dom_fail(b->dom[d], s);
}

int score_batch_restart(score_batch* b) {
    if (!b) return SCORE_ERR_ARG;
    for (score_ctx* c : b->dom) {
        if (!c->a.grid) continue;
        const int s = score_restart(c);
        if (s != SCORE_OK) return b->dom_fail(c, s);
    }
    for (auto& E : b->engs) E->mark_run_start();
    return SCORE_OK;
}

int score_batch_place_nuclei(score_batch* b) {
    if (!b) return SCORE_ERR_ARG;
    for (score_ctx* c : b->dom) {
        if (!c->loaded) continue;
        const int s = score_place_nuclei(c, nullptr);
        if (s != SCORE_OK) return b->dom_fail(c, s);
    }
    return SCORE_OK;
}

int score_batch_run_until(score_batch* b, double x_target, uint32_t max_steps, uint32_t* steps_done) {
    if (!b) return SCORE_ERR_ARG;
    for (score_ctx* c : b->dom) c->trace.clear();
    std::vector<uint32_t> steps(b->engs.size(), 0);
    const int s = b->each_group([&](size_t g) { return b->engs[g]->run_until(x_target, max_steps, &steps[g]); });
    if (steps_done) *steps_done = *std::max_element(steps.begin(), steps.end());
    return s;
}

int score_batch_get_stats(score_batch* b, uint32_t d, score_step_stats* out) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    return score_get_stats(b->dom[d], out);
}

int score_batch_trace(score_batch* b, uint32_t d, score_step_stats* trace, uint32_t cap, uint32_t* n_steps) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    const std::vector<score_step_stats>& t = b->dom[d]->trace;
    if (trace) for (uint32_t i = 0; i < cap && i < t.size(); ++i) trace[i] = t[i];
    if (n_steps) *n_steps = (uint32_t)t.size();
    return SCORE_OK;
}

int score_batch_export_labels(score_batch* b, uint32_t d, uint32_t* labels) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    const int s = score_export_labels(b->dom[d], labels);
    return s == SCORE_OK ? s : b->dom_fail(b->dom[d], s);
}

int score_batch_grain_counts(score_batch* b, uint32_t d, uint32_t* rxg_counts, uint32_t* defg_counts) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    const int s = score_grain_counts(b->dom[d], rxg_counts, defg_counts);
    return s == SCORE_OK ? s : b->dom_fail(b->dom[d], s);
}

int score_batch_grainevo_count(score_batch* b, uint32_t d, uint32_t* n) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    return score_grainevo_count(b->dom[d], n);
}

int score_batch_grainevo(score_batch* b, uint32_t d, uint32_t i, score_grainevo_info* info, uint32_t* counts, uint32_t* rxarea) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    const int s = grainevo_get(b->dom[d], i, info, counts, rxarea);
    return s == SCORE_OK ? s : b->dom_fail(b->dom[d], s);
}

int score_batch_rediscr_kinetics(score_batch* b, uint32_t nslots, double* t_out, double* rxvol_out, double* boxvol_out) {
    if (!b) return SCORE_ERR_ARG;
    return rediscr(b->dom, nslots, nullptr, 0, t_out, rxvol_out, boxvol_out, b->err);
}

int score_batch_rediscr_texture(score_batch* b, uint32_t nslots, const uint32_t* grain_class, uint32_t nclass, double* t_out,
                                double* vol_out) {
    if (!b || !grain_class) return SCORE_ERR_ARG;
    size_t n = 0;
    for (score_ctx* c : b->dom) n += (size_t)c->ndefg + c->nrxg;
    for (size_t i = 0; i < n; ++i)
        if (grain_class[i] >= nclass) return b->fail(SCORE_ERR_ARG, "orientation class out of range");
    return rediscr(b->dom, nslots, grain_class, nclass, t_out, vol_out, nullptr, b->err);
}

int score_batch_final_grain_sizes(score_batch* b, uint32_t* rx_cells) {
    if (!b || !rx_cells) return SCORE_ERR_ARG;
    size_t off = 0;
    for (score_ctx* c : b->dom) {
        if (!c->loaded) return b->fail(SCORE_ERR_STATE, "every domain must be loaded");
        cudaSetDevice(c->device);
        cudaError_t e = c->nrxg ? cudaMemcpyAsync(rx_cells + off, c->a.rxg_cnt, (size_t)c->nrxg * 4, cudaMemcpyDeviceToHost, c->stream)
                                : cudaSuccess;
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return b->fail(SCORE_ERR_CUDA, std::string("final grain sizes: ") + cudaGetErrorString(e));
        off += c->nrxg;
    }
    return SCORE_OK;
}

int score_batch_percolation_analyze(score_batch* b, uint32_t d, int mode, score_perc_result* out, uint32_t* sizes, uint32_t sizes_cap,
                            uint32_t* labels) {
    if (!b || d >= b->dom.size()) return SCORE_ERR_ARG;
    const int s = score_percolation_analyze(b->dom[d], mode, out, sizes, sizes_cap, labels);
    return s == SCORE_OK ? s : b->dom_fail(b->dom[d], s);
}

int score_batch_get_timing(score_batch* b, score_timing* out) {
    if (!b || !out) return SCORE_ERR_ARG;
    // device and host times summed over the groups (they run concurrently), the run span the longest
    *out = score_timing{};
    uint64_t launches = 0;
    for (auto& E : b->engs) {
        const score_timing& t = E->tm;
        out->total_ms += t.total_ms; out->grow_ms += t.grow_ms; out->claim_ms += t.claim_ms; out->commit_ms += t.commit_ms;
        out->host_ms += t.host_ms; out->grow_launches += t.grow_launches; out->grow_bytes += t.grow_bytes;
        out->step_bytes += t.step_bytes; out->fill_ms += t.fill_ms; out->wait_ms += t.wait_ms; out->weights_ms += t.weights_ms;
        out->pre_ms += t.pre_ms; out->post_ms += t.post_ms; out->timed_steps += t.timed_steps;
        out->run_ms = std::max(out->run_ms, t.run_ms);
        launches += E->launches;
    }
    for (score_ctx* c : b->dom) launches += c->launches;
    out->kernel_launches = launches;
    return SCORE_OK;
}

int score_batch_get_tune(score_batch* b, score_tune* out) {
    if (!b || !out) return SCORE_ERR_ARG;
    b->engs[0]->get_tune(out);
    return SCORE_OK;
}

int score_batch_set_tune(score_batch* b, const score_tune* t) {
    if (!b || !t) return SCORE_ERR_ARG;
    for (auto& E : b->engs) {
        const int s = E->set_tune(t);
        if (s != SCORE_OK) return b->fail(s, E->err);
    }
    return SCORE_OK;
}

int score_batch_autotune(score_batch* b, double x_target, uint32_t max_steps, score_tune* out) {
    if (!b) return SCORE_ERR_ARG;
    int s = score_batch_restart(b);
    if (s == SCORE_OK) s = score_batch_place_nuclei(b);
    if (s != SCORE_OK) return s;
    std::vector<score_tune> tunes(b->engs.size());
    s = b->each_group([&](size_t g) { return b->engs[g]->autotune(x_target, max_steps, &tunes[g]); });
    if (s != SCORE_OK) return s;
    if (out) *out = tunes[0];
    s = score_batch_restart(b);
    if (s == SCORE_OK) s = score_batch_place_nuclei(b);
    return s;
}

}  // extern "C"

// ------------------------------------------------------------------ no-allocation table
// Device FP64 mobility-weight table P(rxg, defg) for all pairs, with the grid-wide
// maximum, in a form that allocates no memory: the only scratch is the file-scope
// static device array below, whose address is resolved once per device.
//
// The table is the reference's formula (SCORE_Kernel.cpp:2460-2527: Sebald-Gottstein
// -1 / 0 / cos^2 near 40deg<111>, or the Rollett-Holm sigmoid) evaluated with CUDA's
// FP64 math functions (acos, cos, exp, pow) instead of the host libm, so entries agree
// with score_mobility_weight to a few ulp; pairs whose disorientation lies within a
// few ulp of a class threshold (15 deg, 10 deg from 40deg<111>) can land in the other
// class.  The growth step itself does not use this table: it keeps the host's values.
namespace {

// Static scratch of the entry point: 256 B of header + one word per table row.
//   word 0          blocks of the current launch that have finished.  Cleared on the
//                   stream before every launch (a launch that was cut short could leave
//                   it non-zero), and set back to 0 by the last block of each launch.
//   words 32 .. 32 + nrxg - 1   maximum P of each row (FP64 bits), written before read.
constexpr uint32_t kTableMaxRows = 65536;
constexpr uint32_t kTableHeaderWords = 32;
static __device__ __align__(256) unsigned long long g_table_scratch[kTableHeaderWords + kTableMaxRows];  // 512 KiB + 256 B

struct TableArgs {
    int32_t model;                  // SCORE_MOBILITY_*
    double fac, lagb, maxdev, m40[4];
    double rh_cut, rh_trans, rh_expo;
};

__device__ double d_weight(const DomainArgs& A, const TableArgs& t, const double pr[4], const double qd[4]) {
    // the 24 Grimmer candidates once: their largest |component| gives the disorientation
    // angle and, for the Sebald-Gottstein weight, the candidate whose axis is compared
    // with 40deg<111>
    double c[6][4];
    d_grimmer(A, pr, qd, c);
    int mi = 0;
    double om = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (fabs(c[i][j]) > om) { om = fabs(c[i][j]); mi = i; }
    const double theta = om < (1.0 - 5.0e-16) ? 2.0 * acos(om) : 0.0;
    if (t.model == SCORE_MOBILITY_ROLLETT_HOLM)
        return 1.0 - (t.rh_cut * exp(-1.0 * t.rh_trans * pow(theta / t.lagb, t.rh_expo)));
    if (theta <= t.lagb) return -1.0;
    // disorientation quaternion of the best symmetry candidate, components sorted descending
    double s[4] = {fabs(c[mi][0]), fabs(c[mi][1]), fabs(c[mi][2]), fabs(c[mi][3])};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3 - i; ++k)
            if (s[k] > s[k + 1]) { const double x = s[k]; s[k] = s[k + 1]; s[k + 1] = x; }
    const double qdis[4] = {s[3], s[2], s[1], s[0]};
    const double dev = d_disori(A, qdis, t.m40, nullptr);
    if (dev < t.maxdev) {
        const double cs = cos(0.5 * kPi * dev / t.maxdev);
        return cs * cs;
    }
    return 0.0;
}

// one block per row rxg; the last block to finish reduces the row maxima
__global__ void __launch_bounds__(256) k_mobility_table(TableArgs t, const double* __restrict__ rxq, uint32_t nrxg,
                                                        const double* __restrict__ dfq, uint32_t ndefg,
                                                        double* __restrict__ table, double* __restrict__ pmax,
                                                        unsigned long long* scratch) {
    DomainArgs A{};
    A.pc_fac = t.fac;
    __shared__ double s_max[8];
    __shared__ bool s_last;
    const uint32_t row = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double pr[4] = {rxq[4 * (size_t)row], rxq[4 * (size_t)row + 1], rxq[4 * (size_t)row + 2], rxq[4 * (size_t)row + 3]};
    double m = -HUGE_VAL;
    for (uint32_t j = threadIdx.x; j < ndefg; j += blockDim.x) {
        const double qd[4] = {dfq[4 * (size_t)j], dfq[4 * (size_t)j + 1], dfq[4 * (size_t)j + 2], dfq[4 * (size_t)j + 3]};
        const double P = d_weight(A, t, pr, qd);
        table[(size_t)row * ndefg + j] = P;
        m = fmax(m, P);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if (lane == 0) s_max[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double bm = s_max[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) bm = fmax(bm, s_max[w]);
        scratch[kTableHeaderWords + row] = (unsigned long long)__double_as_longlong(bm);
        __threadfence();
        const unsigned long long done = atomicAdd(&scratch[0], 1ull);
        s_last = (done == (unsigned long long)nrxg - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double g = -HUGE_VAL;
    for (uint32_t r = threadIdx.x; r < nrxg; r += blockDim.x)
        g = fmax(g, __longlong_as_double((long long)__ldcg(&scratch[kTableHeaderWords + r])));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g = fmax(g, __shfl_xor_sync(0xFFFFFFFFu, g, o));
    if (lane == 0) s_max[warp] = g;
    __syncthreads();
    if (threadIdx.x == 0) {
        double bm = s_max[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) bm = fmax(bm, s_max[w]);
        *pmax = bm;
        scratch[0] = 0ull;  // ready for the next launch
    }
}

// scratch address per device ordinal, resolved once with that device current
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned long long* g_scratch_of[kMaxDevices] = {};

int table_scratch(int device, unsigned long long** out) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_of[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_table_scratch);
        if (e != cudaSuccess || !p) return SCORE_ERR_CUDA;
        g_scratch_of[device] = (unsigned long long*)p;
    }
    *out = g_scratch_of[device];
    return SCORE_OK;
}

}  // namespace

extern "C" int score_mobility_table_noalloc(const score_params* p, const double* d_rxg_quat, uint32_t nrxg,
                                            const double* d_defg_quat, uint32_t ndefg, double* d_table,
                                            double* d_pmax, void* stream) {
    if (!p || !d_rxg_quat || !d_defg_quat || !d_table || !d_pmax || nrxg == 0 || ndefg == 0) return SCORE_ERR_ARG;
    if (nrxg > kTableMaxRows) return SCORE_ERR_SCRATCH_LIMIT;
    if (p->mobility_model != SCORE_MOBILITY_SEBALD_GOTTSTEIN && p->mobility_model != SCORE_MOBILITY_ROLLETT_HOLM)
        return SCORE_ERR_ARG;
    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0) return SCORE_ERR_NOT_BUILT;
    if (device >= kMaxDevices) return SCORE_ERR_ARG;
    unsigned long long* scratch = nullptr;
    const int s = table_scratch(device, &scratch);
    if (s != SCORE_OK) return s;
    TableArgs t{};
    t.model = p->mobility_model;
    double theta_sat = 0.0;
    weight_constants(*p, &t.fac, &t.lagb, &t.maxdev, t.m40, &theta_sat);
    t.rh_cut = p->RH_cut;
    t.rh_trans = p->RH_trans;
    t.rh_expo = p->RH_exponent;
    cudaStream_t st = (cudaStream_t)stream;
    // the completion counter starts at 0 whatever an earlier launch left behind
    if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), st) != cudaSuccess) return SCORE_ERR_CUDA;
    // the launch's own status (not cudaGetLastError, which would also report, and clear,
    // an error left behind by the caller's earlier work)
    void* args[] = {(void*)&t, (void*)&d_rxg_quat, (void*)&nrxg, (void*)&d_defg_quat, (void*)&ndefg, (void*)&d_table,
                    (void*)&d_pmax, (void*)&scratch};
    const cudaError_t e = cudaLaunchKernel((const void*)k_mobility_table, dim3(nrxg), dim3(256), args, 0, st);
    return e == cudaSuccess ? SCORE_OK : SCORE_ERR_CUDA;
}
