// sm_103a kernels of one recrystallization growth step.
//
// GB300 executes FP64 at 1/64 of the FP32 rate, so the bit-exact FP64 path keeps
// FP64 instructions off the per-update critical path.  Every front cell stores
//   vel = (m(P) * p(defg)) * f_geo(infector)      (the reference's first three roundings)
//   inc = (vel * dt) * (1/cellsize)               (its fill increment for the current dt)
// Both are computed when the cell is infected (with that step's dt); vel again only when
// T, rho or the drag change, inc only when dt changed or for a cell whose vel was not
// known at infection (a nucleus, or a weight the host computes: kStale bit of the
// infector byte).  A typical update is then one DADD,
//   fill = fill + inc,
// with the "fill >= 1" test on the integer bit pattern (fill is never negative).
// A cell whose driving force is <= 5e-16 stores vel = inc = -1 and is skipped, as the
// reference skips it (calcGrowthStepInside, SCORE_Kernel.cpp:4046-4130).
//
// Every ordered compaction (FullRX list, recycle list, slot ranks of new cells) is a
// count pass that also adds its counts into supertile sums, and a write pass that
// takes each tile's exclusive prefix from the supertile and tile counts: no block
// ever waits on another one.
//   k_grow_fill   per list: fill update of every ACTIVE slot in [0, next_never);
//                 1-bit masks of full and INACTIVE slots, per-warp counts; Sv count.
//   k_grow_lists  FullRX list and capped recycle list, in slot order.
//   k_claim   one thread per full cell: the 26 infection attempts in the reference's
//             order; a still-deformed target gets atomicMin(claim, attempt ordinal),
//             where ordinal = 26 * (full-cell rank, Inside list first) + direction rank.
//             The thread records which attempts it made (26-bit mask).
//   k_resolve one thread per full cell: attempts whose claim holds the own ordinal
//             won; per-tile win counts per destination list.
//   k_commit  winners are ranked per destination list in full-cell then direction
//             order and take recycled slots first, then appended slots, like
//             omp_getNextFreeSlotInRXFront*(CELLRECYCLE).  The full cell then becomes
//             recrystallized (grid = ndefg + rxg, counts, slot INACTIVE) — the tail of
//             updateFullRX{Inside,Border}, SCORE_Kernel.cpp:4559-4774.  The wins of a
//             tile are spread over all its threads; each new cell gets its mobility
//             weight P (from the table, or a tag for the host) and cached velocity
//             factor.
//   k_step_end  slot high-water marks, stats snapshot, reset of the per-step fields.
#pragma once
#include <cstdint>
#include "device_common.cuh"

namespace score {

struct DFront {
    void* fill;          // double (FP64) or float (FP32)
    float* comp;         // Kahan compensation (FP32 only)
    void* vel;           // double (FP64) or float (FP32): (m p) f_geo, or -1 = no driving force
    double* inc;         // FP64 only: cached (vel dt) / cellsize for the current dt
    double* mob;         // cached mobility m(P) of the cell's boundary (a refresh when only p changed)
    uint32_t* defg;
    uint32_t* rxg;
    uint32_t* xyz;       // linear cell index x + y nx + z nx ny
    uint8_t* dir;        // infector code 0..26 (| kStale), kInactive = INACTIVE
    uint32_t* full;      // FullRX list (slot indices, slot order)
    uint32_t* recyc;     // recycle list (slot indices, slot order, capped)
    uint32_t* fmask;     // per 32 slots: full slots of this step (bit = slot % 32)
    uint32_t* imask;     // per 32 slots: INACTIVE slots of this step
    uint32_t* tcnt;      // per warp of a grow tile: (full, INACTIVE) counts
    uint32_t* scnt;      // per supertile of kSuper grow tiles: the same counts (zero between steps)
    uint32_t cap;        // device capacity of the slot arrays
    uint32_t reccap;     // ntotalRecyclingList of the reference
};

// n / d for n < 2^31 by multiply-high (Granlund-Montgomery), d >= 1
struct FastDiv {
    uint32_t d, mul, shr;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f{d, 0u, 0u};
    if (d > 1) {
        uint32_t l = 0;
        while ((1ull << l) < d) ++l;  // ceil(log2 d)
        const uint32_t p = 31 + l;
        f.mul = (uint32_t)(((1ull << p) + d - 1) / d);
        f.shr = p - 32;
    }
    return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return f.d == 1 ? n : (__umulhi(n, f.mul) >> f.shr);
}

struct HostBox;

struct DomainArgs {
    DFront f[2];
    DevState* st;
    uint32_t* grid;             // grain id per cell, in 2x2x2 bricks (gindex)
    uint32_t* claim;            // lowest attempt ordinal per cell this step, same layout
    uint32_t* amask;            // per full cell: attempts made (bit d), then attempts won
    uint32_t* tobm;             // per full cell: won attempts that go to the Border list
    uint32_t* fcell;            // per full cell: its cell (brick index, written by k_claim)
    uint32_t* ctcnt;            // per commit tile: (Inside, Border) win counts
    uint32_t* csct;             // per supertile of kSuper commit tiles: the same counts (zero between steps)
    unsigned long long* ptab;   // nrxg x ndefg mobility weights as bits (kPtabEmpty = unknown)
    const double* pforce;       // per deformed grain driving force (FP64)
    uint32_t* defg_cnt;
    uint32_t* rxg_cnt;
    uint32_t* depleted;
    unsigned long long* miss;   // table indices the host must fill
    uint32_t misscap;
    uint32_t nx, ny, nz;
    uint32_t gbx, gby, gbxy;    // bricks along x, along y, per brick layer
    uint32_t ncells;            // grid words: 8 per brick, the domain padded to even extents
    FastDiv dgbx, dgbxy;
    uint32_t ndefg, nrxg;
    uint32_t border_ref_cap;
    int32_t border_policy, boundary, mobility_model;
    int32_t dt_changed;         // dt differs from the dt the cached increments were made with
    int32_t refresh;            // recompute every vel this step: 1 from P (mobilities changed), 2 from the
                                // cached mobility (only the driving force changed), 0 no
    int32_t active;             // the domain steps in this launch
    const unsigned long long* ans_idx;  // weights the host computed for the last step's requests, in miss-slot
                                        // order: table indices (kMissVoid = none), device view of pinned memory
    const double* ans_val;
    HostBox* box;               // device view of the domain's mailbox
    double mLAGB, mHAGB, mGS, mRH, dt, cinv;
    float dtc32;
    int32_t spec;               // few INACTIVE slots last step: k_grow_fill loads every slot's data with its
                                // infector byte instead of only the ACTIVE slots' (no effect on results)
    double pc_fac;              // 1/sqrt(2) as the host computes it (the disorientation of d_grimmer)
};

// Cells on the device are named by their grid word: the grid is stored in bricks of 2x2x2 cells
// (8 consecutive words, x fastest inside the brick), bricks in x, then y, then z order, so that
// the 3x3x3 neighbourhood of any cell lies in 8 bricks, one 32-byte sector each.  Front slots,
// full-cell positions and nucleus sites hold this brick index; the linear index x + nx (y + ny z)
// of the C interface is converted at the boundary (load, labels).
__host__ __device__ __forceinline__ uint32_t gindex(uint32_t gbx, uint32_t gby, uint32_t x, uint32_t y, uint32_t z) {
    return ((((z >> 1) * gby + (y >> 1)) * gbx + (x >> 1)) << 3) | ((z & 1u) << 2) | ((y & 1u) << 1) | (x & 1u);
}
__device__ __forceinline__ uint32_t gindex(const DomainArgs& a, uint32_t x, uint32_t y, uint32_t z) {
    return gindex(a.gbx, a.gby, x, y, z);
}

__device__ __forceinline__ void decode(const DomainArgs& a, uint32_t cell, int& x, int& y, int& z) {
    const uint32_t b = cell >> 3;
    const uint32_t bz = fdiv(b, a.dgbxy);
    const uint32_t r = b - bz * a.gbxy;
    const uint32_t by = fdiv(r, a.dgbx);
    x = (int)(2u * (r - by * a.gbx) + (cell & 1u));
    y = (int)(2u * by + ((cell >> 1) & 1u));
    z = (int)(2u * bz + ((cell >> 2) & 1u));
}

// linear index of the C interface
__device__ __forceinline__ uint32_t linear_of(const DomainArgs& a, int x, int y, int z) {
    return (uint32_t)x + a.nx * ((uint32_t)y + a.ny * (uint32_t)z);
}

// Target of attempt d from (x,y,z) of a cell of list L.  Inside cells are strictly
// interior so their neighbours need no wrap; Border cells wrap x,y periodically and
// drop z (reference) or wrap z (periodic build option).  false = attempt dropped.
__device__ __forceinline__ bool target_of(const DomainArgs& a, int L, int x, int y, int z, int d, uint32_t& t, bool& interior) {
    int tx = x + c_dx[d], ty = y + c_dy[d], tz = z + c_dz[d];
    if (L == 1) {
        if (tx < 0) tx += (int)a.nx;
        if (tx >= (int)a.nx) tx -= (int)a.nx;
        if (ty < 0) ty += (int)a.ny;
        if (ty >= (int)a.ny) ty -= (int)a.ny;
        if (a.boundary == 0) {
            if (tz < 0 || tz >= (int)a.nz) return false;
        } else {
            if (tz < 0) tz += (int)a.nz;
            if (tz >= (int)a.nz) tz -= (int)a.nz;
        }
    } else if (tx < 0 || ty < 0 || tz < 0 || tx >= (int)a.nx || ty >= (int)a.ny || tz >= (int)a.nz) {
        atomicOr(&a.st->err, kErrBounds);
        return false;
    }
    interior = tx > 0 && tx < (int)a.nx - 1 && ty > 0 && ty < (int)a.ny - 1 && tz > 0 && tz < (int)a.nz - 1;
    t = gindex(a, (uint32_t)tx, (uint32_t)ty, (uint32_t)tz);
    return true;
}

// mobility m(P) of the reference (get_currentintrinsicmobility, SCORE_Kernel.cpp:5459-5470)
__device__ __forceinline__ double mobility(const DomainArgs& a, double P) {
    if (a.mobility_model == 2) return __dmul_rn(P, a.mRH);
    if (P < 0.0) return a.mLAGB;
    return __dadd_rn(__dmul_rn(P, a.mGS), __dmul_rn(__dsub_rn(1.0, P), a.mHAGB));
}
// velocity factor (m p) f_geo, or -1 when the driving force is not above 5e-16
__device__ __forceinline__ double velocity_from_force(double m, double p, int code) {
    if (!(p > 5.0e-16)) return -1.0;
    return __dmul_rn(__dmul_rn(m, p), c_sf[code]);
}
__device__ __forceinline__ double velocity_from_mobility(const DomainArgs& a, double m, uint32_t defg, int code) {
    return velocity_from_force(m, a.pforce[defg], code);
}
__device__ __forceinline__ double velocity_factor(const DomainArgs& a, double P, uint32_t defg, int code) {
    return velocity_from_mobility(a, mobility(a, P), defg, code);
}

// warp-0 exclusive scan of 2x64 block-local counters laid out [item][warp]; totals in every lane
__device__ __forceinline__ void scan64_pair(uint32_t* cntA, uint32_t* cntB, uint32_t& totA, uint32_t& totB) {
    const int lane = threadIdx.x & 31;
    uint32_t a0 = cntA[2 * lane], a1 = cntA[2 * lane + 1], b0 = cntB[2 * lane], b1 = cntB[2 * lane + 1];
    uint32_t as = a0 + a1, bs = b0 + b1, ai = as, bi = bs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t x = __shfl_up_sync(0xFFFFFFFFu, ai, o), y = __shfl_up_sync(0xFFFFFFFFu, bi, o);
        if (lane >= o) { ai += x; bi += y; }
    }
    uint32_t ae = ai - as, be = bi - bs;
    cntA[2 * lane] = ae; cntA[2 * lane + 1] = ae + a0;
    cntB[2 * lane] = be; cntB[2 * lane + 1] = be + b0;
    totA = __shfl_sync(0xFFFFFFFFu, ai, 31);
    totB = __shfl_sync(0xFFFFFFFFu, bi, 31);
}

// ------------------------------------------------------------------ work over many domains
// Every step kernel takes the array of per-domain argument blocks and walks a global
// list of work units (tiles, full cells, new cells) that concatenates the domains'
// (and lists') units; a block first builds the exclusive prefix of the unit counts of
// all segments in shared memory and maps a unit to its segment by binary search.
// One domain is the batch of size one.
constexpr int kMaxDomains = 64;
constexpr int kMaxSegs = 2 * kMaxDomains;

// Argument blocks of every domain that steps on this device, in constant memory: a
// field read is a constant-cache access that stores never invalidate.  Each engine
// owns a range of slots; its kernels take the range's base.
__constant__ DomainArgs c_args[kMaxDomains];

// Block-wide (kBlock threads) exclusive scan of the unit counts of `nseg` segments
// into s_pre[0..nseg]; count(seg) is evaluated once per segment.  Returns the total.
template <class Count>
__device__ __forceinline__ uint32_t seg_prefix(uint32_t* s_pre, int nseg, Count count) {
    __shared__ uint32_t s_warp[kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int PER = (kMaxSegs + kBlock - 1) / kBlock;  // segments per thread
    uint32_t v[PER], sum = 0;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int s = threadIdx.x * PER + j;
        v[j] = s < nseg ? count(s) : 0u;
        sum += v[j];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += x;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        before += w < warp ? s_warp[w] : 0u;
        total += s_warp[w];
    }
    uint32_t e = before + inc - sum;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int s = threadIdx.x * PER + j;
        if (s < nseg) s_pre[s] = e;
        e += v[j];
    }
    if (threadIdx.x == 0) s_pre[nseg] = total;
    __syncthreads();
    return total;
}

// segment of unit u: the last s with s_pre[s] <= u (segments with no units are skipped)
__device__ __forceinline__ int seg_find(const uint32_t* s_pre, int nseg, uint32_t u) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_pre[mid] <= u) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Thread-per-item kernels pad each segment to whole warps, so that the 32 items of a
// warp belong to one domain and its argument reads stay uniform (one constant-cache
// access per field); padding items are skipped.
__device__ __forceinline__ uint32_t warp_pad(uint32_t n) { return (n + 31u) & ~31u; }

// grow tiles of a list: kBlock * ITEMS slots, ITEMS * kWarps mask words
template <int ITEMS>
struct GrowShape {
    static constexpr uint32_t kTile = kBlock * ITEMS;
    static constexpr uint32_t kWords = ITEMS * kWarps;
};
constexpr uint32_t kSuper = 64;  // tiles per supertile of the two-level tile prefix

// Exclusive prefix of tile `tile` of a (cnt: count pairs, `per` entries per tile;
// sup: per-supertile pairs) count array, computed by one warp; every lane returns both.
template <int U = 4>
__device__ __forceinline__ void tile_prefix(const uint32_t* cnt, const uint32_t* sup, uint32_t tile, uint32_t& pa, uint32_t& pb,
                                            uint32_t per = 1) {
    // the supertile sums [0, s) then the count pairs [s kSuper per, tile per), as one
    // index range of 8-byte loads with U in flight per lane before any add waits
    const uint32_t s = tile / kSuper, lo = s * kSuper * per, n = s + (tile * per - lo);
    const uint2* ps = (const uint2*)sup;
    const uint2* pc = (const uint2*)cnt + lo - s;
    uint32_t a = 0, b = 0;
    for (uint32_t i = threadIdx.x & 31; i < n; i += 32 * U) {
        uint2 x[U];
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const uint32_t j = i + 32u * k;
            x[k] = j < n ? (j < s ? ps[j] : pc[j]) : make_uint2(0u, 0u);
        }
#pragma unroll
        for (int k = 0; k < U; ++k) { a += x[k].x; b += x[k].y; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
        b += __shfl_xor_sync(0xFFFFFFFFu, b, o);
    }
    pa = a; pb = b;
}

// ------------------------------------------------------------------ K1 grow
// Two launches, neither of which waits on another block:
//   k_grow_fill   streams the slots of every (domain, list) in tiles of kBlock*ITEMS
//                 slots, updates the fills, writes one bit per slot (full / INACTIVE)
//                 and the tile's two counts, and adds them to its supertile's counts;
//   k_grow_lists  one warp per tile: the tile's exclusive prefix from the supertile
//                 and tile counts, then the FullRX list and the capped recycle list in
//                 slot order; the warp of a list's last tile stores the list totals.
// REFRESH 1: recompute vel of every active slot from the P table and the current physics
// (after T changed the mobilities); REFRESH 2: from the cell's cached mobility (only rho or the
// drag changed the driving force), no table gather; REFRESH 0: the cached increment (or vel when
// dt changed or the increment is stale); REFRESH 3: as 0 with dt unchanged when the last step's
// list had few holes: every slot's data is loaded with its infector byte, whether ACTIVE or not
// (one memory round trip instead of two).
// A cell created last step whose weight the host computed: P = answer `tag`; the table
// entry (tagged until now) gets the value for later lookups.
__device__ __forceinline__ double answered_velocity(const DomainArgs& a, const DFront& fr, uint32_t slot, uint8_t dir,
                                                    unsigned long long tag) {
    const uint32_t m = (uint32_t)tag;
    const double P = a.ans_val[m];
    a.ptab[a.ans_idx[m]] = (unsigned long long)__double_as_longlong(P);
    const double mo = mobility(a, P);
    fr.mob[slot] = mo;
    return velocity_from_mobility(a, mo, fr.defg[slot], dir & kCodeMask);
}

// The full and INACTIVE masks of a warp's ITEMS x 32 slots of grow tile `tile` (slot of item k and
// lane: base + 32 k), the warp's two counts and its share of the supertile's counts.
template <int ITEMS>
__device__ __forceinline__ void tile_masks(const DFront& fr, uint32_t tile, uint32_t base, uint32_t n, uint32_t act, uint32_t fullbits) {
    using S = GrowShape<ITEMS>;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t word0 = tile * S::kWords + (uint32_t)(warp * ITEMS);  // item k's mask word
    uint32_t cf = 0, ci = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const uint32_t fm = __ballot_sync(0xFFFFFFFFu, (fullbits >> k) & 1u);
        const uint32_t im = __ballot_sync(0xFFFFFFFFu, !((act >> k) & 1u) && base + (uint32_t)(k * 32) < n);
        if (lane == 0) {
            const uint32_t word = word0 + (uint32_t)k;  // slots 32 word .. 32 word + 31
            fr.fmask[word] = fm;
            fr.imask[word] = im;
        }
        cf += __popc(fm);
        ci += __popc(im);
    }
    if (lane == 0) {  // the warp's counts, and its share of the supertile's
        const uint32_t wt = tile * kWarps + (uint32_t)warp;
        fr.tcnt[2 * wt] = cf;
        fr.tcnt[2 * wt + 1] = ci;
        if (cf) atomicAdd(&fr.scnt[2 * (tile / kSuper)], cf);
        if (ci) atomicAdd(&fr.scnt[2 * (tile / kSuper) + 1], ci);
    }
}

// returns the thread's ACTIVE slots (the Sv share)
template <bool FP32, int REFRESH, int ITEMS>
__device__ __forceinline__ uint32_t grow_tile(const DomainArgs& a, int L, uint32_t tile, uint32_t n) {
    using S = GrowShape<ITEMS>;
    const DFront& fr = a.f[L];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // each warp owns 32 * ITEMS consecutive slots of the tile: no block barrier, warps run apart
    const uint32_t base = tile * S::kTile + (uint32_t)warp * 32u * ITEMS + (uint32_t)lane;
    uint32_t sv = 0, act = 0;  // act bit k: item k's slot is ACTIVE
    uint8_t d[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const uint32_t slot = base + (uint32_t)(k * 32);
        d[k] = slot < n ? fr.dir[slot] : kInactive;
        if (d[k] != kInactive) act |= 1u << k;
    }
    uint32_t fullbits = 0;  // bit k: item k's cell is full
    if (!FP32 && REFRESH == 3) {
        double w[ITEMS], fill[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t slot = base + (uint32_t)(k * 32);
            w[k] = -1.0; fill[k] = 0.0;
            if (slot < n) {
                w[k] = fr.inc[slot];
                fill[k] = ((const double*)fr.fill)[slot];
            }
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t slot = base + (uint32_t)(k * 32);
            if (((act >> k) & 1u) && (d[k] & kStale)) {
                if (d[k] & kPend) {
                    w[k] = answered_velocity(a, fr, slot, d[k], ((const unsigned long long*)fr.vel)[slot]);
                    ((double*)fr.vel)[slot] = w[k];
                } else {
                    w[k] = ((const double*)fr.vel)[slot];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (!((act >> k) & 1u)) continue;
            ++sv;
            const uint32_t slot = base + (uint32_t)(k * 32);
            double inc = w[k];
            if (d[k] & kStale) {
                if (__double_as_longlong(w[k]) >= 0) inc = __dmul_rn(__dmul_rn(w[k], a.dt), a.cinv);
                fr.inc[slot] = inc;
                fr.dir[slot] = d[k] & kCodeMask;
            }
            if (__double_as_longlong(inc) >= 0) {
                const double f = __dadd_rn(fill[k], inc);
                ((double*)fr.fill)[slot] = f;
                if (__double_as_longlong(f) >= 0x3FF0000000000000ll) fullbits |= 1u << k;
            }
        }
    } else if (!FP32) {
        // in two halves of the items, each loaded, brought to its velocity factor and updated before
        // the next: the loads of one half stay in flight together and nothing spills
        constexpr int H = ITEMS / 2;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            double w[H], fill[H];  // w: cached inc, or vel when the increment is stale
            if (REFRESH == 0) {
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    w[j] = -1.0; fill[j] = 0.0;
                    if ((act >> k) & 1u) {
                        w[j] = a.dt_changed ? ((const double*)fr.vel)[slot] : fr.inc[slot];
                        fill[j] = ((const double*)fr.fill)[slot];
                    }
                }
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    if (((act >> k) & 1u) && (d[k] & kStale)) {  // nuclei, cells answered by the host: no increment yet
                        if (d[k] & kPend) {
                            w[j] = answered_velocity(a, fr, slot, d[k], ((const unsigned long long*)fr.vel)[slot]);
                            ((double*)fr.vel)[slot] = w[j];
                        } else if (!a.dt_changed) {
                            w[j] = ((const double*)fr.vel)[slot];
                        }
                    }
                }
            } else if (REFRESH == 2) {
                double mo[H];
                uint32_t g[H];
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    w[j] = -1.0; fill[j] = 0.0; mo[j] = 0.0; g[j] = 0;
                    if ((act >> k) & 1u) {
                        mo[j] = fr.mob[slot];
                        g[j] = fr.defg[slot];
                        fill[j] = ((const double*)fr.fill)[slot];
                    }
                }
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    if ((act >> k) & 1u) {
                        if (d[k] & kPend) w[j] = answered_velocity(a, fr, slot, d[k], ((const unsigned long long*)fr.vel)[slot]);
                        else w[j] = velocity_from_mobility(a, mo[j], g[j], d[k] & kCodeMask);
                        ((double*)fr.vel)[slot] = w[j];
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    w[j] = -1.0; fill[j] = 0.0;
                    if ((act >> k) & 1u) {
                        if (d[k] & kPend) {
                            w[j] = answered_velocity(a, fr, slot, d[k], ((const unsigned long long*)fr.vel)[slot]);
                        } else {
                            const uint32_t g = fr.defg[slot];
                            const double P = __longlong_as_double((long long)a.ptab[(unsigned long long)fr.rxg[slot] * a.ndefg + g]);
                            const double mo = mobility(a, P);
                            fr.mob[slot] = mo;
                            w[j] = velocity_from_mobility(a, mo, g, d[k] & kCodeMask);
                        }
                        ((double*)fr.vel)[slot] = w[j];
                        fill[j] = ((const double*)fr.fill)[slot];
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < H; ++j) {
                const int k = h * H + j;
                if (!((act >> k) & 1u)) continue;
                ++sv;
                const uint32_t slot = base + (uint32_t)(k * 32);
                double inc = w[j];
                if (REFRESH != 0 || a.dt_changed || (d[k] & kStale)) {
                    if (__double_as_longlong(w[j]) >= 0) inc = __dmul_rn(__dmul_rn(w[j], a.dt), a.cinv);
                    fr.inc[slot] = inc;
                    if (d[k] & kStale) fr.dir[slot] = d[k] & kCodeMask;
                }
                if (__double_as_longlong(inc) >= 0) {  // sign bit clear: driving force present
                    const double f = __dadd_rn(fill[j], inc);
                    ((double*)fr.fill)[slot] = f;
                    if (__double_as_longlong(f) >= 0x3FF0000000000000ll) fullbits |= 1u << k;  // f >= 1.0, never negative
                }
            }
        }
    } else {
        constexpr int H = ITEMS / 2;  // two halves, as the FP64 fill
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float vel[H], fill[H], comp[H];
            if (REFRESH == 0 || REFRESH == 3) {
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    vel[j] = -1.0f; fill[j] = 0.0f; comp[j] = 0.0f;
                    if (REFRESH == 3 ? slot < n : ((act >> k) & 1u)) {
                        vel[j] = ((const float*)fr.vel)[slot];
                        fill[j] = ((const float*)fr.fill)[slot];
                        comp[j] = fr.comp[slot];
                    }
                }
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    if (((act >> k) & 1u) && (d[k] & kPend)) {
                        vel[j] = (float)answered_velocity(a, fr, slot, d[k], ((const uint32_t*)fr.vel)[slot]);
                        ((float*)fr.vel)[slot] = vel[j];
                    }
                }
            } else if (REFRESH == 2) {
                double mo[H];
                uint32_t g[H];
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    vel[j] = -1.0f; fill[j] = 0.0f; comp[j] = 0.0f; mo[j] = 0.0; g[j] = 0;
                    if ((act >> k) & 1u) {
                        mo[j] = fr.mob[slot];
                        g[j] = fr.defg[slot];
                        fill[j] = ((const float*)fr.fill)[slot];
                        comp[j] = fr.comp[slot];
                    }
                }
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    if ((act >> k) & 1u) {
                        if (d[k] & kPend) vel[j] = (float)answered_velocity(a, fr, slot, d[k], ((const uint32_t*)fr.vel)[slot]);
                        else vel[j] = (float)velocity_from_mobility(a, mo[j], g[j], d[k] & kCodeMask);
                        ((float*)fr.vel)[slot] = vel[j];
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const int k = h * H + j;
                    const uint32_t slot = base + (uint32_t)(k * 32);
                    vel[j] = -1.0f; fill[j] = 0.0f; comp[j] = 0.0f;
                    if ((act >> k) & 1u) {
                        if (d[k] & kPend) {
                            vel[j] = (float)answered_velocity(a, fr, slot, d[k], ((const uint32_t*)fr.vel)[slot]);
                        } else {
                            const uint32_t g = fr.defg[slot];
                            const double P = __longlong_as_double((long long)a.ptab[(unsigned long long)fr.rxg[slot] * a.ndefg + g]);
                            const double mo = mobility(a, P);
                            fr.mob[slot] = mo;
                            vel[j] = (float)velocity_from_mobility(a, mo, g, d[k] & kCodeMask);
                        }
                        ((float*)fr.vel)[slot] = vel[j];
                        fill[j] = ((const float*)fr.fill)[slot];
                        comp[j] = fr.comp[slot];
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < H; ++j) {
                const int k = h * H + j;
                if (!((act >> k) & 1u)) continue;
                ++sv;
                const uint32_t slot = base + (uint32_t)(k * 32);
                if (d[k] & kStale) fr.dir[slot] = d[k] & kCodeMask;
                if (vel[j] >= 0.0f) {
                    // Kahan-compensated accumulation of the fill
                    const float inc = vel[j] * a.dtc32;
                    const float y = inc - comp[j];
                    const float t = fill[j] + y;
                    const float c = (t - fill[j]) - y;
                    ((float*)fr.fill)[slot] = t;
                    fr.comp[slot] = c;
                    if ((t - c) >= 1.0f) fullbits |= 1u << k;
                }
            }
        }
    }
    tile_masks<ITEMS>(fr, tile, base, n, act, fullbits);
    return sv;
}

// warp-summed Sv share into the domain's counter (one atomic per warp and segment)
__device__ __forceinline__ void flush_sv(const DomainArgs& a, int L, uint32_t sv) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sv += __shfl_xor_sync(0xFFFFFFFFu, sv, o);
    if ((threadIdx.x & 31) == 0 && sv) atomicAdd(&a.st->sv[L], (unsigned long long)sv);
}

// a single domain's Sv shares of the whole block into its counters: one atomic per list and block
// (a per-warp atomic on the same two words from every block of a launch serialises at the end)
__device__ __forceinline__ void flush_sv_block(const DomainArgs& a, uint32_t sv0, uint32_t sv1) {
    __shared__ uint32_t s_sv[2][kWarps];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sv0 += __shfl_xor_sync(0xFFFFFFFFu, sv0, o);
        sv1 += __shfl_xor_sync(0xFFFFFFFFu, sv1, o);
    }
    if ((threadIdx.x & 31) == 0) { s_sv[0][threadIdx.x >> 5] = sv0; s_sv[1][threadIdx.x >> 5] = sv1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t0 = 0, t1 = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) { t0 += s_sv[0][w]; t1 += s_sv[1][w]; }
        if (t0) atomicAdd(&a.st->sv[0], (unsigned long long)t0);
        if (t1) atomicAdd(&a.st->sv[1], (unsigned long long)t1);
    }
}

// slots of list L of a domain this step ( 0 for a domain that is not stepping)
__device__ __forceinline__ uint32_t list_slots(const DomainArgs& a, int L) { return a.active ? a.st->next_never[L] : 0u; }

// ONE: a single domain (the plain path): its argument block sits at a launch-uniform
// slot and the two lists are walked in turn, so every argument read is uniform.
// MODE: the grow mode every stepping domain uses this step (0, 1, 2, 3 as grow_tile's REFRESH), or
// kFillAny to decide per domain.  The host knows a single domain's mode before the launch, and a
// kernel specialised to one mode holds only that mode's loads in its registers.
constexpr int kFillAny = -1;

template <bool FP32, int ITEMS, int MODE>
__device__ __forceinline__ uint32_t grow_tile_mode(const DomainArgs& a, int L, uint32_t tile, uint32_t n) {
    if (MODE == kFillAny) {
        if (a.refresh == 2) return grow_tile<FP32, 2, ITEMS>(a, L, tile, n);
        if (a.refresh == 1) return grow_tile<FP32, 1, ITEMS>(a, L, tile, n);
        if (a.spec && !a.dt_changed) return grow_tile<FP32, 3, ITEMS>(a, L, tile, n);
        return grow_tile<FP32, 0, ITEMS>(a, L, tile, n);
    }
    return grow_tile<FP32, MODE == kFillAny ? 0 : MODE, ITEMS>(a, L, tile, n);
}

template <bool FP32, int ITEMS, bool ONE, int MODE>
__global__ void __launch_bounds__(kBlock, ITEMS >= 16 ? 2 : 4) k_grow_fill(int base, int ndom) {
    using S = GrowShape<ITEMS>;
    __shared__ uint32_t s_pre[kMaxSegs + 1];
    if (ONE) {
        const DomainArgs& a = c_args[base];
        if (!a.active) return;
        uint32_t sv[2] = {0, 0};
#pragma unroll
        for (int L = 0; L < 2; ++L) {
            const uint32_t n = a.st->next_never[L];
            const uint32_t ntiles = (n + S::kTile - 1) / S::kTile;
            for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) sv[L] += grow_tile_mode<FP32, ITEMS, MODE>(a, L, tile, n);
        }
        flush_sv_block(a, sv[0], sv[1]);
        return;
    }
    const int nseg = 2 * ndom;
    const uint32_t total = seg_prefix(s_pre, nseg, [&](int s) {
        return (list_slots(c_args[base + (s >> 1)], s & 1) + S::kTile - 1) / S::kTile;
    });
    int cur = -1;       // segment whose Sv share is being accumulated
    uint32_t sv = 0;
    for (uint32_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int s = seg_find(s_pre, nseg, u);
        if (s != cur) {
            if (cur >= 0) flush_sv(c_args[base + (cur >> 1)], cur & 1, sv);
            cur = s;
            sv = 0;
        }
        const DomainArgs& a = c_args[base + (s >> 1)];
        const int L = s & 1;
        const uint32_t tile = u - s_pre[s];
        sv += grow_tile_mode<FP32, ITEMS, MODE>(a, L, tile, a.st->next_never[L]);
    }
    if (cur >= 0) flush_sv(c_args[base + (cur >> 1)], cur & 1, sv);
}

// The FP64 fill of a single domain in grow mode 3 (dt unchanged, few holes), software-pipelined:
// a thread's loads for its next tile (infector bytes, increments, fills) are issued before the
// current tile's additions, so that one tile's FP64 adds and stores overlap the next tile's memory
// round trip.  The tiles of both lists form one sequence (list 0's, then list 1's).  Arithmetic,
// stores and masks are grow_tile's in mode 3.
template <int ITEMS>
struct Mode3Regs {
    uint8_t d[ITEMS];
    double w[ITEMS], f[ITEMS];
};

template <int ITEMS>
__device__ __forceinline__ void mode3_load(const DomainArgs& a, uint32_t u, uint32_t t0, uint32_t n0, uint32_t n1, Mode3Regs<ITEMS>& r) {
    using S = GrowShape<ITEMS>;
    const int L = u >= t0 ? 1 : 0;
    const DFront& fr = a.f[L];
    const uint32_t n = L ? n1 : n0;
    const uint32_t base = (L ? u - t0 : u) * S::kTile + (uint32_t)(threadIdx.x >> 5) * 32u * ITEMS + (threadIdx.x & 31u);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const uint32_t slot = base + (uint32_t)(k * 32);
        r.d[k] = kInactive; r.w[k] = -1.0; r.f[k] = 0.0;
        if (slot < n) {
            r.d[k] = fr.dir[slot];
            r.w[k] = fr.inc[slot];
            r.f[k] = ((const double*)fr.fill)[slot];
        }
    }
}

template <int ITEMS>
__global__ void __launch_bounds__(kBlock, ITEMS >= 8 ? 2 : 3) k_grow_fill_pf(int base) {
    using S = GrowShape<ITEMS>;
    const DomainArgs& a = c_args[base];
    if (!a.active) return;
    const uint32_t n0 = a.st->next_never[0], n1 = a.st->next_never[1];
    const uint32_t t0 = (n0 + S::kTile - 1) / S::kTile, total = t0 + (n1 + S::kTile - 1) / S::kTile;
    uint32_t sv0 = 0, sv1 = 0;  // ACTIVE slots per list
    uint32_t u = blockIdx.x;
    Mode3Regs<ITEMS> cur;
    if (u < total) mode3_load<ITEMS>(a, u, t0, n0, n1, cur);
    while (u < total) {
        const uint32_t un = u + gridDim.x;
        Mode3Regs<ITEMS> nxt;
        if (un < total) mode3_load<ITEMS>(a, un, t0, n0, n1, nxt);  // in flight during this tile's work
        const int L = u >= t0 ? 1 : 0;
        const DFront& fr = a.f[L];
        const uint32_t n = L ? n1 : n0, tile = L ? u - t0 : u;
        const uint32_t base_slot = tile * S::kTile + (uint32_t)(threadIdx.x >> 5) * 32u * ITEMS + (threadIdx.x & 31u);
        uint32_t act = 0, fullbits = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (cur.d[k] == kInactive) continue;
            act |= 1u << k;
            if (!(cur.d[k] & kStale)) continue;  // nuclei, cells answered by the host: no increment yet
            const uint32_t slot = base_slot + (uint32_t)(k * 32);
            double w;
            if (cur.d[k] & kPend) {
                w = answered_velocity(a, fr, slot, cur.d[k], ((const unsigned long long*)fr.vel)[slot]);
                ((double*)fr.vel)[slot] = w;
            } else {
                w = ((const double*)fr.vel)[slot];
            }
            cur.w[k] = __double_as_longlong(w) >= 0 ? __dmul_rn(__dmul_rn(w, a.dt), a.cinv) : w;
            fr.inc[slot] = cur.w[k];
            fr.dir[slot] = cur.d[k] & kCodeMask;
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            // sign bit clear: driving force present
            if (!((act >> k) & 1u) || __double_as_longlong(cur.w[k]) < 0) continue;
            const double f = __dadd_rn(cur.f[k], cur.w[k]);
            ((double*)fr.fill)[base_slot + (uint32_t)(k * 32)] = f;
            if (__double_as_longlong(f) >= 0x3FF0000000000000ll) fullbits |= 1u << k;  // f >= 1.0
        }
        if (L) sv1 += (uint32_t)__popc(act);
        else sv0 += (uint32_t)__popc(act);
        tile_masks<ITEMS>(fr, tile, base_slot, n, act, fullbits);
        u = un;
        if (u < total) cur = nxt;
    }
    flush_sv_block(a, sv0, sv1);
}

// The FP64 fill of a single domain in grow mode 0 (the cached increment, or vel when dt changed;
// lists with many holes, so only ACTIVE slots' data is loaded), pipelined over a thread's tiles: the
// next tile's infector bytes are in flight while this tile's increments and fills are loaded, added
// and stored, so that a tile costs one memory round trip instead of two.  Arithmetic, stores and
// masks are grow_tile's in mode 0.
template <int ITEMS>
__device__ __forceinline__ void mode0_dir(const DomainArgs& a, uint32_t u, uint32_t t0, uint32_t n0, uint32_t n1, uint8_t (&d)[ITEMS]) {
    using S = GrowShape<ITEMS>;
    const int L = u >= t0 ? 1 : 0;
    const uint32_t n = L ? n1 : n0;
    const uint32_t base = (L ? u - t0 : u) * S::kTile + (uint32_t)(threadIdx.x >> 5) * 32u * ITEMS + (threadIdx.x & 31u);
    const uint8_t* dir = a.f[L].dir;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const uint32_t slot = base + (uint32_t)(k * 32);
        d[k] = slot < n ? dir[slot] : kInactive;
    }
}

template <int ITEMS>
__global__ void __launch_bounds__(kBlock, ITEMS >= 16 ? 2 : 3) k_grow_fill_pf0(int base) {
    using S = GrowShape<ITEMS>;
    const DomainArgs& a = c_args[base];
    if (!a.active) return;
    const uint32_t n0 = a.st->next_never[0], n1 = a.st->next_never[1];
    const uint32_t t0 = (n0 + S::kTile - 1) / S::kTile, total = t0 + (n1 + S::kTile - 1) / S::kTile;
    const bool dtc = a.dt_changed != 0;
    uint32_t sv0 = 0, sv1 = 0;  // ACTIVE slots per list
    uint32_t u = blockIdx.x;
    uint8_t d[ITEMS];
    if (u < total) mode0_dir<ITEMS>(a, u, t0, n0, n1, d);
    while (u < total) {
        const uint32_t un = u + gridDim.x;
        uint8_t dn[ITEMS];
        if (un < total) mode0_dir<ITEMS>(a, un, t0, n0, n1, dn);  // in flight during this tile's work
        const int L = u >= t0 ? 1 : 0;
        const DFront& fr = a.f[L];
        const uint32_t n = L ? n1 : n0, tile = L ? u - t0 : u;
        const uint32_t base_slot = tile * S::kTile + (uint32_t)(threadIdx.x >> 5) * 32u * ITEMS + (threadIdx.x & 31u);
        uint32_t act = 0, fullbits = 0;
        double w[ITEMS], fil[ITEMS];  // w: cached inc, or vel when the increment is stale or dt changed
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t slot = base_slot + (uint32_t)(k * 32);
            w[k] = -1.0; fil[k] = 0.0;
            if (d[k] != kInactive) {
                act |= 1u << k;
                w[k] = dtc ? ((const double*)fr.vel)[slot] : fr.inc[slot];
                fil[k] = ((const double*)fr.fill)[slot];
            }
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (!((act >> k) & 1u) || !(d[k] & kStale)) continue;  // nuclei, cells answered by the host: no increment yet
            const uint32_t slot = base_slot + (uint32_t)(k * 32);
            if (d[k] & kPend) {
                w[k] = answered_velocity(a, fr, slot, d[k], ((const unsigned long long*)fr.vel)[slot]);
                ((double*)fr.vel)[slot] = w[k];
            } else if (!dtc) {
                w[k] = ((const double*)fr.vel)[slot];
            }
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            if (!((act >> k) & 1u)) continue;
            const uint32_t slot = base_slot + (uint32_t)(k * 32);
            double inc = w[k];
            if (dtc || (d[k] & kStale)) {
                if (__double_as_longlong(w[k]) >= 0) inc = __dmul_rn(__dmul_rn(w[k], a.dt), a.cinv);
                fr.inc[slot] = inc;
                if (d[k] & kStale) fr.dir[slot] = d[k] & kCodeMask;
            }
            if (__double_as_longlong(inc) >= 0) {  // sign bit clear: driving force present
                const double f = __dadd_rn(fil[k], inc);
                ((double*)fr.fill)[slot] = f;
                if (__double_as_longlong(f) >= 0x3FF0000000000000ll) fullbits |= 1u << k;  // f >= 1.0
            }
        }
        if (L) sv1 += (uint32_t)__popc(act);
        else sv0 += (uint32_t)__popc(act);
        tile_masks<ITEMS>(fr, tile, base_slot, n, act, fullbits);
        u = un;
        if (u < total) {
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) d[k] = dn[k];
        }
    }
    flush_sv_block(a, sv0, sv1);
}

// The fill of a single domain (FP64, or FP32 + Kahan) in grow mode 0 while most of the list is holes
// (the last step's INACTIVE share above spec_holes_pct).  A block takes a whole grow tile with one vector load of
// infector bytes per thread (ITEMS consecutive slots each); each warp gathers its ACTIVE slots into a
// shared list, and its lanes take them up to 4 x 32 at a time with all their increment and fill
// loads in flight together, so that a memory round trip serves up to 128 ACTIVE slots instead of the
// few a thread's strided items hold.  The next tile's infector bytes are in flight meanwhile.
// Arithmetic and stores are grow_tile's in mode 0; the full and INACTIVE masks and the per-warp
// counts keep the layout k_grow_lists reads.
template <int ITEMS>
struct SparseDir {  // a thread's ITEMS infector bytes
    static_assert(ITEMS == 4 || ITEMS == 8 || ITEMS == 16, "items");
    uint32_t w[ITEMS / 4];
};

// the thread's ITEMS infector bytes of grow tile `tile` of list L (n slots)
template <int ITEMS>
__device__ __forceinline__ void sparse_dir(const DomainArgs& a, int L, uint32_t tile, uint32_t n, SparseDir<ITEMS>& r) {
    using S = GrowShape<ITEMS>;
    const uint32_t first = tile * S::kTile + threadIdx.x * (uint32_t)ITEMS;
    const uint8_t* dir = a.f[L].dir;
    if (first + ITEMS <= n) {  // ITEMS bytes at an ITEMS-aligned slot: one vector load
        if (ITEMS == 4) r.w[0] = *(const uint32_t*)(dir + first);
        else if (ITEMS == 8) { const uint2 v = *(const uint2*)(dir + first); r.w[0] = v.x; r.w[1] = v.y; }
        else { const uint4 v = *(const uint4*)(dir + first); r.w[0] = v.x; r.w[1] = v.y; r.w[2] = v.z; r.w[3] = v.w; }
    } else {
#pragma unroll
        for (int j = 0; j < ITEMS / 4; ++j) r.w[j] = 0xFFFFFFFFu;  // past the list: INACTIVE
        for (uint32_t j = 0; first + j < n && j < (uint32_t)ITEMS; ++j) {
            const uint32_t sh = 8u * (j & 3u);
            r.w[j >> 2] = (r.w[j >> 2] & ~(0xFFu << sh)) | ((uint32_t)dir[first + j] << sh);
        }
    }
}

template <int ITEMS>
struct SparseShared {  // a block's shared lists: per warp its ACTIVE slots, their infector bytes, full bits
    uint32_t slot[kWarps][32 * ITEMS];
    uint8_t dir[kWarps][32 * ITEMS];
    uint32_t full[kWarps][ITEMS];
};

// One grow tile of list L (n slots) by the whole block, the thread's infector bytes in `cur`:
// returns the thread's ACTIVE slots.  Warps run apart (no block barrier).
template <bool FP32, int ITEMS>
__device__ __forceinline__ uint32_t sparse_tile(const DomainArgs& a, int L, uint32_t tile, uint32_t n, const SparseDir<ITEMS>& cur,
                                                SparseShared<ITEMS>& sh) {
    using S = GrowShape<ITEMS>;
    constexpr uint32_t WS = 32u * ITEMS;  // slots of a warp's part of the tile
    constexpr int B = 4;                  // ACTIVE slots per lane with loads in flight together
    uint32_t (&s_slot)[kWarps][WS] = sh.slot;
    uint8_t (&s_dir)[kWarps][WS] = sh.dir;
    uint32_t (&s_full)[kWarps][ITEMS] = sh.full;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const DFront& fr = a.f[L];
    const bool dtc = a.dt_changed != 0;
    const uint32_t wfirst = tile * S::kTile + (uint32_t)warp * WS;  // the warp's first slot
    const uint32_t first = tile * S::kTile + threadIdx.x * (uint32_t)ITEMS;  // the thread's
    uint32_t act = 0;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
        if (((cur.w[j >> 2] >> (8 * (j & 3))) & 0xFFu) != kInactive) act |= 1u << j;
    // the warp's ACTIVE slots into its shared list, in slot order
    const uint32_t c = (uint32_t)__popc(act);
    uint32_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    const uint32_t wcnt = __shfl_sync(0xFFFFFFFFu, x, 31);
    uint32_t pos = x - c;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
        if ((act >> j) & 1u) {
            s_slot[warp][pos] = first + (uint32_t)j;
            s_dir[warp][pos] = (uint8_t)((cur.w[j >> 2] >> (8 * (j & 3))) & 0xFFu);
            ++pos;
        }
    if (lane < ITEMS) s_full[warp][lane] = 0u;
    __syncwarp();
    // the lanes take the warp's ACTIVE slots, B x 32 at a time, all their loads issued first
    for (uint32_t i0 = 0; i0 < wcnt; i0 += 32u * B) {
        uint32_t slot[B];
        uint8_t d[B];
        double w[B], fil[B];  // FP64: cached inc (or vel), fill; FP32: vel, fill
        float cmp[B];         // FP32: Kahan compensation
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const uint32_t i = i0 + 32u * b + (uint32_t)lane;
            d[b] = kInactive; slot[b] = 0; w[b] = -1.0; fil[b] = 0.0; cmp[b] = 0.0f;
            if (i < wcnt) {
                slot[b] = s_slot[warp][i];
                d[b] = s_dir[warp][i];
                if (!FP32) {
                    w[b] = dtc ? ((const double*)fr.vel)[slot[b]] : fr.inc[slot[b]];
                    fil[b] = ((const double*)fr.fill)[slot[b]];
                } else {
                    w[b] = ((const float*)fr.vel)[slot[b]];
                    fil[b] = ((const float*)fr.fill)[slot[b]];
                    cmp[b] = fr.comp[slot[b]];
                }
            }
        }
#pragma unroll
        for (int b = 0; b < B; ++b) {
            if (d[b] == kInactive) continue;
            bool full = false;
            if (!FP32) {
                if (d[b] & kStale) {  // nuclei, cells answered by the host: no increment yet
                    if (d[b] & kPend) {
                        w[b] = answered_velocity(a, fr, slot[b], d[b], ((const unsigned long long*)fr.vel)[slot[b]]);
                        ((double*)fr.vel)[slot[b]] = w[b];
                    } else if (!dtc) {
                        w[b] = ((const double*)fr.vel)[slot[b]];
                    }
                }
                double inc = w[b];
                if (dtc || (d[b] & kStale)) {
                    if (__double_as_longlong(w[b]) >= 0) inc = __dmul_rn(__dmul_rn(w[b], a.dt), a.cinv);
                    fr.inc[slot[b]] = inc;
                    if (d[b] & kStale) fr.dir[slot[b]] = d[b] & kCodeMask;
                }
                if (__double_as_longlong(inc) >= 0) {  // sign bit clear: driving force present
                    const double f = __dadd_rn(fil[b], inc);
                    ((double*)fr.fill)[slot[b]] = f;
                    full = __double_as_longlong(f) >= 0x3FF0000000000000ll;  // f >= 1.0
                }
            } else {
                float vel = (float)w[b];
                if (d[b] & kPend) {  // P from the host
                    vel = (float)answered_velocity(a, fr, slot[b], d[b], ((const uint32_t*)fr.vel)[slot[b]]);
                    ((float*)fr.vel)[slot[b]] = vel;
                }
                if (d[b] & kStale) fr.dir[slot[b]] = d[b] & kCodeMask;
                if (vel >= 0.0f) {
                    // Kahan-compensated accumulation of the fill
                    const float fl = (float)fil[b];
                    const float inc = vel * a.dtc32;
                    const float y = inc - cmp[b];
                    const float t = fl + y;
                    const float c = (t - fl) - y;
                    ((float*)fr.fill)[slot[b]] = t;
                    fr.comp[slot[b]] = c;
                    full = (t - c) >= 1.0f;
                }
            }
            if (full) {
                const uint32_t k = slot[b] - wfirst;
                atomicOr(&s_full[warp][k >> 5], 1u << (k & 31u));
            }
        }
    }
    __syncwarp();
    // the thread's full and INACTIVE bits into the masks: 32 / ITEMS threads share a mask word
    const uint32_t kl = (uint32_t)lane * ITEMS;  // the thread's first slot within the warp's part
    const uint32_t fb = (s_full[warp][kl >> 5] >> (kl & 31u)) & ((1u << ITEMS) - 1u);
    uint32_t ib = ~act & ((1u << ITEMS) - 1u);
    if (first + ITEMS > n) ib &= first >= n ? 0u : ((1u << (n - first)) - 1u);  // slots past the list are not INACTIVE
    uint32_t fm = fb << (kl & 31u), im = ib << (kl & 31u);
#pragma unroll
    for (int o = 1; o < 32 / ITEMS; o <<= 1) {
        fm |= __shfl_xor_sync(0xFFFFFFFFu, fm, o);
        im |= __shfl_xor_sync(0xFFFFFFFFu, im, o);
    }
    if ((kl & 31u) == 0u) {
        fr.fmask[first >> 5] = fm;  // slots 32 word .. 32 word + 31
        fr.imask[first >> 5] = im;
    }
    uint32_t cf = (uint32_t)__popc(fb), ci = (uint32_t)__popc(ib);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cf += __shfl_xor_sync(0xFFFFFFFFu, cf, o);
        ci += __shfl_xor_sync(0xFFFFFFFFu, ci, o);
    }
    if (lane == 0) {  // the warp's counts, and its share of the supertile's
        const uint32_t wt = tile * kWarps + (uint32_t)warp;
        fr.tcnt[2 * wt] = cf;
        fr.tcnt[2 * wt + 1] = ci;
        if (cf) atomicAdd(&fr.scnt[2 * (tile / kSuper)], cf);
        if (ci) atomicAdd(&fr.scnt[2 * (tile / kSuper) + 1], ci);
    }
    __syncwarp();  // the shared list is rewritten by the next tile
    return c;
}

template <bool FP32, int ITEMS>
__global__ void __launch_bounds__(kBlock, 4) k_grow_fill_sparse(int base) {
    using S = GrowShape<ITEMS>;
    __shared__ SparseShared<ITEMS> sh;
    const DomainArgs& a = c_args[base];
    if (!a.active) return;
    const uint32_t n0 = a.st->next_never[0], n1 = a.st->next_never[1];
    const uint32_t t0 = (n0 + S::kTile - 1) / S::kTile, total = t0 + (n1 + S::kTile - 1) / S::kTile;
    uint32_t sv0 = 0, sv1 = 0;  // ACTIVE slots per list
    uint32_t u = blockIdx.x;
    SparseDir<ITEMS> cur;
    if (u < total) sparse_dir<ITEMS>(a, u >= t0 ? 1 : 0, u >= t0 ? u - t0 : u, u >= t0 ? n1 : n0, cur);
    while (u < total) {
        const uint32_t un = u + gridDim.x;
        SparseDir<ITEMS> nxt;
        if (un < total) sparse_dir<ITEMS>(a, un >= t0 ? 1 : 0, un >= t0 ? un - t0 : un, un >= t0 ? n1 : n0, nxt);  // in flight meanwhile
        const int L = u >= t0 ? 1 : 0;
        const uint32_t c = sparse_tile<FP32, ITEMS>(a, L, L ? u - t0 : u, L ? n1 : n0, cur, sh);
        if (L) sv1 += c;
        else sv0 += c;
        u = un;
        if (u < total) cur = nxt;
    }
    flush_sv_block(a, sv0, sv1);
}

// The same for a batch whose domains all step from cached increments (no refresh this step): the
// grow tiles of every (domain, list) form one sequence, mapped to their segment by binary search.
template <bool FP32, int ITEMS>
__global__ void __launch_bounds__(kBlock, 4) k_grow_fill_sparse_batch(int base, int ndom) {
    using S = GrowShape<ITEMS>;
    __shared__ SparseShared<ITEMS> sh;
    __shared__ uint32_t s_pre[kMaxSegs + 1];
    const int nseg = 2 * ndom;
    const uint32_t total = seg_prefix(s_pre, nseg, [&](int s) {
        return (list_slots(c_args[base + (s >> 1)], s & 1) + S::kTile - 1) / S::kTile;
    });
    auto locate = [&](uint32_t v, int& s, uint32_t& tile) { s = seg_find(s_pre, nseg, v); tile = v - s_pre[s]; };
    int cur_seg = -1;   // segment whose Sv share is being accumulated
    uint32_t sv = 0;
    uint32_t u = blockIdx.x;
    SparseDir<ITEMS> cur;
    if (u < total) {
        int s; uint32_t t;
        locate(u, s, t);
        sparse_dir<ITEMS>(c_args[base + (s >> 1)], s & 1, t, c_args[base + (s >> 1)].st->next_never[s & 1], cur);
    }
    while (u < total) {
        const uint32_t un = u + gridDim.x;
        SparseDir<ITEMS> nxt;
        if (un < total) {
            int s; uint32_t t;
            locate(un, s, t);
            sparse_dir<ITEMS>(c_args[base + (s >> 1)], s & 1, t, c_args[base + (s >> 1)].st->next_never[s & 1], nxt);
        }
        int s; uint32_t tile;
        locate(u, s, tile);
        if (s != cur_seg) {
            if (cur_seg >= 0) flush_sv(c_args[base + (cur_seg >> 1)], cur_seg & 1, sv);
            cur_seg = s;
            sv = 0;
        }
        const DomainArgs& a = c_args[base + (s >> 1)];
        sv += sparse_tile<FP32, ITEMS>(a, s & 1, tile, a.st->next_never[s & 1], cur, sh);
        u = un;
        if (u < total) cur = nxt;
    }
    if (cur_seg >= 0) flush_sv(c_args[base + (cur_seg >> 1)], cur_seg & 1, sv);
}

// one warp per grow tile
template <int ITEMS>
__global__ void __launch_bounds__(kBlock) k_grow_lists(int base, int ndom) {
    using S = GrowShape<ITEMS>;
    constexpr int WPL = (int)S::kWords / 32;  // mask words per lane
    __shared__ uint32_t s_pre[kMaxSegs + 1];
    const int nseg = 2 * ndom;
    const uint32_t total = seg_prefix(s_pre, nseg, [&](int s) {
        return (list_slots(c_args[base + (s >> 1)], s & 1) + S::kTile - 1) / S::kTile;
    });
    const int lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < total; u += nw) {
        const int s = seg_find(s_pre, nseg, u);
        const DomainArgs& a = c_args[base + (s >> 1)];
        const int L = s & 1;
        const DFront& fr = a.f[L];
        const uint32_t tile = u - s_pre[s];
        uint32_t rf, ri;
        // the fill wrote one count pair per warp: up to kSuper x kWarps pairs, all loads in flight at once
        tile_prefix<8>(fr.tcnt, fr.scnt, tile, rf, ri, kWarps);
        uint32_t fw[WPL], iw[WPL];
#pragma unroll
        for (int h = 0; h < WPL; ++h) {
            fw[h] = fr.fmask[tile * S::kWords + (uint32_t)(32 * h + lane)];
            iw[h] = fr.imask[tile * S::kWords + (uint32_t)(32 * h + lane)];
        }
        const uint32_t reccap = fr.reccap;
#pragma unroll
        for (int h = 0; h < WPL; ++h) {
            uint32_t cf = __popc(fw[h]), ci = __popc(iw[h]);
            uint32_t xf = cf, xi = ci;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t p = __shfl_up_sync(0xFFFFFFFFu, xf, o), q = __shfl_up_sync(0xFFFFFFFFu, xi, o);
                if (lane >= o) { xf += p; xi += q; }
            }
            // lane j owns word 32h + j of the tile: slots tile kTile + 32 (32h + j) + bit
            const uint32_t wslot = tile * S::kTile + 32u * (uint32_t)(32 * h + lane);
            // full slots are a few per cent of the slots: each lane writes its word's, in bit order
            uint32_t r = rf + xf - cf;
            for (uint32_t m = fw[h]; m; m &= m - 1u) fr.full[r++] = wslot + (uint32_t)(__ffs(m) - 1);
            // INACTIVE slots only up to the recycle cap (SCORE_Kernel.cpp:4133-4180); the rest are not listed.
            // Dense words go through the warp in word order so that the stores coalesce.
            uint32_t q0 = ri + xi - ci;
            if (__any_sync(0xFFFFFFFFu, q0 < reccap && ci)) {
                if (__ballot_sync(0xFFFFFFFFu, ci > 8u)) {
                    for (int j = 0; j < 32; ++j) {
                        const uint32_t wi = __shfl_sync(0xFFFFFFFFu, iw[h], j), bi = __shfl_sync(0xFFFFFFFFu, q0, j);
                        if (bi >= reccap || !wi) continue;  // uniform over the warp
                        if ((wi >> lane) & 1u) {
                            const uint32_t rr = bi + __popc(wi & lt);
                            if (rr < reccap) fr.recyc[rr] = tile * S::kTile + 32u * (uint32_t)(32 * h + j) + (uint32_t)lane;
                        }
                    }
                } else {
                    for (uint32_t m = iw[h]; m && q0 < reccap; m &= m - 1u) fr.recyc[q0++] = wslot + (uint32_t)(__ffs(m) - 1);
                }
            }
            rf += __shfl_sync(0xFFFFFFFFu, xf, 31);
            ri += __shfl_sync(0xFFFFFFFFu, xi, 31);
        }
        if (tile + 1 == s_pre[s + 1] - s_pre[s] && lane == 0) {  // the list's last tile: totals
            a.st->nfull[L] = rf;
            a.st->ninactive[L] = ri;
            a.st->nrec[L] = min(ri, reccap);
        }
    }
}

constexpr int kGrowItems = 8;                        // tile shape of the defragmentation passes
constexpr uint32_t kGrowTile = kBlock * kGrowItems;

// In-place exclusive scan of `ntiles` (a, b) count pairs by one block of 1024 threads;
// returns the totals in thread 0.
__device__ __forceinline__ void scan_pairs_block(uint32_t* cnt, uint32_t ntiles, uint32_t& totA, uint32_t& totB) {
    constexpr int T = 1024, PER = 4;
    __shared__ uint32_t s_a[T / 32], s_b[T / 32];
    __shared__ uint32_t s_carry[2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) { s_carry[0] = 0; s_carry[1] = 0; }
    __syncthreads();
    for (uint32_t base = 0; base < ntiles; base += T * PER) {
        uint32_t va[PER], vb[PER], sa = 0, sb = 0;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const uint32_t i = base + threadIdx.x * PER + j;
            va[j] = i < ntiles ? cnt[2 * i] : 0u;
            vb[j] = i < ntiles ? cnt[2 * i + 1] : 0u;
            sa += va[j]; sb += vb[j];
        }
        uint32_t ia = sa, ib = sb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t xa = __shfl_up_sync(0xFFFFFFFFu, ia, o), xb = __shfl_up_sync(0xFFFFFFFFu, ib, o);
            if (lane >= o) { ia += xa; ib += xb; }
        }
        if (lane == 31) { s_a[warp] = ia; s_b[warp] = ib; }
        __syncthreads();
        if (warp == 0) {
            uint32_t wa = s_a[lane], wb = s_b[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t xa = __shfl_up_sync(0xFFFFFFFFu, wa, o), xb = __shfl_up_sync(0xFFFFFFFFu, wb, o);
                if (lane >= o) { wa += xa; wb += xb; }
            }
            s_a[lane] = wa; s_b[lane] = wb;  // inclusive warp prefixes
        }
        __syncthreads();
        uint32_t ea = s_carry[0] + (warp ? s_a[warp - 1] : 0u) + ia - sa;
        uint32_t eb = s_carry[1] + (warp ? s_b[warp - 1] : 0u) + ib - sb;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const uint32_t i = base + threadIdx.x * PER + j;
            if (i < ntiles) { cnt[2 * i] = ea; cnt[2 * i + 1] = eb; }
            ea += va[j]; eb += vb[j];
        }
        __syncthreads();
        if (threadIdx.x == 0) { s_carry[0] += s_a[31]; s_carry[1] += s_b[31]; }
        __syncthreads();
    }
    totA = s_carry[0];
    totB = s_carry[1];
}

// ------------------------------------------------------------------ K2 claim
// Attempts LO..HI-1 of one Border cell: the grid loads are all issued before the atomics
// (claims are a min, so the order of the atomics does not matter); targets wrap through target_of.
template <int LO, int HI>
__device__ __forceinline__ uint32_t claim_plane(const DomainArgs& a, int x, int y, int z, uint32_t f) {
    uint32_t tg[HI - LO], gv[HI - LO];
#pragma unroll
    for (int k = 0; k < HI - LO; ++k) {
        gv[k] = 0xFFFFFFFFu;
        bool inter;
        if (target_of(a, 1, x, y, z, LO + k, tg[k], inter)) gv[k] = a.grid[tg[k]];
    }
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < HI - LO; ++k) {
        if (gv[k] < a.ndefg) {
            atomicMin(&a.claim[tg[k]], f * 26u + (uint32_t)(LO + k));
            mask |= 1u << (LO + k);
        }
    }
    return mask;
}

// full cells of a domain this step (Inside list first); 0 when the 32-bit attempt
// ordinal 26 f + d could overflow (flagged)
__device__ __forceinline__ uint32_t full_cells(const DomainArgs& a) {
    if (!a.active) return 0u;
    const uint32_t F = a.st->nfull[0] + a.st->nfull[1];
    return 26ull * F >= 0xFFFFFFFFull ? 0u : F;
}

template <bool ONE>
__global__ void __launch_bounds__(kBlock, 2) k_claim(int base, int ndom) {
    __shared__ uint32_t s_pre[kMaxSegs + 1], s_cnt[kMaxSegs];
    auto count = [&](int s) {
        const DomainArgs& a = c_args[base + (s)];
        if (a.active && 26ull * (a.st->nfull[0] + a.st->nfull[1]) >= 0xFFFFFFFFull) atomicOr(&a.st->err, kErrKeyLimit);
        return full_cells(a);
    };
    uint32_t total;
    if (ONE) {
        total = count(0);
    } else {
        total = seg_prefix(s_pre, ndom, [&](int s) {
            s_cnt[s] = count(s);
            return warp_pad(s_cnt[s]);
        });
    }
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < total; u += gridDim.x * blockDim.x) {
        const int s = ONE ? 0 : seg_find(s_pre, ndom, u);
        const DomainArgs& a = c_args[base + (s)];
        const uint32_t f = ONE ? u : u - s_pre[s];
        if (!ONE && f >= s_cnt[s]) continue;
        const uint32_t F0 = a.st->nfull[0];
        uint32_t mask;
        if (f < F0) {
            // an Inside cell (strictly interior, every list insertion checks it): its neighbourhood
            // spans 8 bricks; all 26 grid reads in flight before the first claim
            const uint32_t cell = a.f[0].xyz[a.f[0].full[f]];
            a.fcell[f] = cell;
            int x, y, z;
            decode(a, cell, x, y, z);
            uint32_t gv[26];
#pragma unroll
            for (int d = 0; d < 26; ++d) {
                const uint32_t t = gindex(a, (uint32_t)(x + c_dx[d]), (uint32_t)(y + c_dy[d]), (uint32_t)(z + c_dz[d]));
                gv[d] = t < a.ncells ? a.grid[t] : 0xFFFFFFFFu;
            }
            mask = 0;
#pragma unroll
            for (int d = 0; d < 26; ++d) {
                const uint32_t t = gindex(a, (uint32_t)(x + c_dx[d]), (uint32_t)(y + c_dy[d]), (uint32_t)(z + c_dz[d]));
                if (t >= a.ncells) atomicOr(&a.st->err, kErrBounds);
                else if (gv[d] < a.ndefg) {
                    atomicMin(&a.claim[t], f * 26u + (uint32_t)d);
                    mask |= 1u << d;
                }
            }
        } else {
            const uint32_t cell = a.f[1].xyz[a.f[1].full[f - F0]];
            a.fcell[f] = cell;
            int x, y, z;
            decode(a, cell, x, y, z);
            mask = claim_plane<0, 8>(a, x, y, z, f);
            mask |= claim_plane<8, 17>(a, x, y, z, f);
            mask |= claim_plane<17, 26>(a, x, y, z, f);
        }
        a.amask[f] = mask;
    }
}

// ---- device disorientation (the no-allocation weight table) ----
// The disorientation's scalar part omega in the host's exact operation sequence (no FMA),
// so only acos differs between device and host libm (a few ulp).
__device__ __forceinline__ void d_quat_mul(const double a[4], const double b[4], double r[4]) {
    r[0] = __dsub_rn(__dsub_rn(__dsub_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2])), __dmul_rn(a[3], b[3]));
    r[1] = __dadd_rn(__dadd_rn(__dmul_rn(b[0], a[1]), __dmul_rn(a[0], b[1])), __dsub_rn(__dmul_rn(a[2], b[3]), __dmul_rn(a[3], b[2])));
    r[2] = __dadd_rn(__dadd_rn(__dmul_rn(b[0], a[2]), __dmul_rn(a[0], b[2])), __dadd_rn(-__dmul_rn(a[1], b[3]), __dmul_rn(a[3], b[1])));
    r[3] = __dadd_rn(__dadd_rn(__dmul_rn(b[0], a[3]), __dmul_rn(a[0], b[3])), __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1])));
}
// the 24 Grimmer candidates (6 quaternions), same order and roundings as the host
__device__ __forceinline__ void d_grimmer(const DomainArgs& A, const double p[4], const double q[4], double c[6][4]) {
    const double qi[4] = {q[0], -q[1], -q[2], -q[3]};
    double r[4];
    d_quat_mul(qi, p, r);
    const double a = r[0], b = r[1], cc = r[2], d = r[3], f = A.pc_fac;
    c[0][0] = __dmul_rn(__dadd_rn(a, b), f);  c[0][1] = __dmul_rn(__dsub_rn(a, b), f);  c[0][2] = __dmul_rn(__dadd_rn(cc, d), f); c[0][3] = __dmul_rn(__dsub_rn(cc, d), f);
    c[1][0] = __dmul_rn(__dadd_rn(a, cc), f); c[1][1] = __dmul_rn(__dsub_rn(a, cc), f); c[1][2] = __dmul_rn(__dadd_rn(b, d), f);  c[1][3] = __dmul_rn(__dsub_rn(b, d), f);
    c[2][0] = __dmul_rn(__dadd_rn(a, d), f);  c[2][1] = __dmul_rn(__dsub_rn(a, d), f);  c[2][2] = __dmul_rn(__dadd_rn(b, cc), f); c[2][3] = __dmul_rn(__dsub_rn(b, cc), f);
    c[3][0] = __dmul_rn(__dadd_rn(__dadd_rn(__dadd_rn(a, b), cc), d), 0.5); c[3][1] = __dmul_rn(__dsub_rn(__dsub_rn(__dadd_rn(a, b), cc), d), 0.5);
    c[3][2] = __dmul_rn(__dsub_rn(__dadd_rn(__dsub_rn(a, b), cc), d), 0.5); c[3][3] = __dmul_rn(__dadd_rn(__dsub_rn(__dsub_rn(a, b), cc), d), 0.5);
    c[4][0] = __dmul_rn(__dsub_rn(__dadd_rn(__dadd_rn(a, b), cc), d), 0.5); c[4][1] = __dmul_rn(__dadd_rn(__dsub_rn(__dadd_rn(a, b), cc), d), 0.5);
    c[4][2] = __dmul_rn(__dadd_rn(__dadd_rn(__dsub_rn(a, b), cc), d), 0.5); c[4][3] = __dmul_rn(__dsub_rn(__dsub_rn(__dsub_rn(a, b), cc), d), 0.5);
    c[5][0] = a; c[5][1] = b; c[5][2] = cc; c[5][3] = d;
}
// disorientation angle; `exact_zero` when the host also returns exactly 0
__device__ __forceinline__ double d_disori(const DomainArgs& A, const double p[4], const double q[4], int* mi_out) {
    double c[6][4];
    d_grimmer(A, p, q, c);
    double om = 0.0;
    int mi = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (fabs(c[i][j]) > om) { om = fabs(c[i][j]); mi = i; }
    if (mi_out) *mi_out = mi;
    if (om < (1.0 - 5.0e-16)) return 2.0 * acos(om);
    return 0.0;
}
// P of a new cell from the table.  An unknown entry is requested from the host (FP64,
// libm, on its worker threads): the first requester takes miss slot m (atomicAdd) and
// tags the entry kPtabTag | m; every cell of the pair carries m and gets P from the host's
// answer m in the next step's k_grow_fill.  A requester that loses the race to tag the
// entry voids its slot.  Returns true with P, or false with the tag.  (Classifying the
// exact-constant weights on the device cost more than it saved: FP64 runs at 1/64 rate,
// cells racing on a new pair all classify it, and the classifier's registers took a
// quarter of this kernel's occupancy.)
__device__ __forceinline__ bool lookup_p(const DomainArgs& a, uint32_t rxg, uint32_t defg, double& P, uint32_t& tag) {
    const unsigned long long idx = (unsigned long long)rxg * a.ndefg + defg;
    unsigned long long* e = &a.ptab[idx];
    // a plain (L1-cached) load: within a launch an entry only goes from EMPTY to a tag, and a stale
    // EMPTY is settled by the compare-and-swap below
    unsigned long long bits = *e;
    if (bits == kPtabEmpty) {
        const uint32_t m = atomicAdd(&a.st->nmiss, 1u);
        if (m >= a.misscap) { atomicOr(&a.st->err, kErrMissCap); tag = 0; return false; }
        const unsigned long long old = atomicCAS(e, kPtabEmpty, kPtabTag | m);
        if (old == kPtabEmpty) {
            a.miss[m] = idx;
            tag = m;
            return false;
        }
        a.miss[m] = kMissVoid;
        bits = old;
    }
    if ((bits >> 48) == (kPtabTag >> 48)) { tag = (uint32_t)bits; return false; }
    P = __longlong_as_double((long long)bits);
    return true;
}

// ------------------------------------------------------------------ K4 step end
// Host mailbox in pinned, device-mapped memory: k_step_end writes the step's scalars,
// the mobility-weight requests and the depleted grains straight into host memory, so
// the host needs one stream synchronization per step and no copies.
constexpr uint32_t kBoxMiss = 16384;
constexpr uint32_t kBoxDep = 16384;
struct HostBox {
    DevState snap;
    unsigned long long miss[kBoxMiss];
    uint32_t depleted[kBoxDep];
};

// The end of a domain's step, by one block: advances the high-water marks, posts the step to the
// domain's mailbox, clears the supertile counters the step used and the per-step fields.  The
// step's scalars, requests and depleted grains are read through L2 (__ldcg): in the commit's last
// block they were written by other blocks of the same launch.
__device__ __forceinline__ void step_end_block(const DomainArgs& a, uint32_t grow_tile) {
    DevState* st = a.st;
    HostBox* box = a.box;
    __shared__ uint32_t s_nm, s_nd, s_sup[3];
    __shared__ unsigned long long s_state[(sizeof(DevState) + 7) / 8];  // the step's scalars, read once through L2
    for (uint32_t i = threadIdx.x; i < sizeof(DevState) / 8; i += blockDim.x) s_state[i] = __ldcg((const unsigned long long*)st + i);
    __syncthreads();
    if (threadIdx.x == 0) {
        DevState& v = *(DevState*)s_state;
        const uint32_t F = v.nfull[0] + v.nfull[1];
        for (int L = 0; L < 2; ++L) s_sup[L] = ((v.next_never[L] + grow_tile - 1) / grow_tile + kSuper - 1) / kSuper;
        s_sup[2] = ((F + kBlock - 1) / kBlock + kSuper - 1) / kSuper;
        const uint32_t cap[2] = {a.f[0].cap, a.f[1].cap};
        for (int D = 0; D < 2; ++D) {
            if (v.nwin[D] > v.nrec[D]) v.next_never[D] += v.nwin[D] - v.nrec[D];
            if (v.next_never[D] > cap[D]) { v.next_never[D] = cap[D]; v.err |= kErrCapacity; }
        }
        st->next_never[0] = v.next_never[0];
        st->next_never[1] = v.next_never[1];
        st->err = v.err;
        box->snap = v;
        s_nm = min(min(v.nmiss, a.misscap), kBoxMiss);
        s_nd = min(min(v.ndepleted, a.ndefg), kBoxDep);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < s_nm; i += blockDim.x) box->miss[i] = __ldcg(&a.miss[i]);
    for (uint32_t i = threadIdx.x; i < s_nd; i += blockDim.x) box->depleted[i] = __ldcg(&a.depleted[i]);
    for (uint32_t i = threadIdx.x; i < 2 * s_sup[0]; i += blockDim.x) a.f[0].scnt[i] = 0u;
    for (uint32_t i = threadIdx.x; i < 2 * s_sup[1]; i += blockDim.x) a.f[1].scnt[i] = 0u;
    for (uint32_t i = threadIdx.x; i < 2 * s_sup[2]; i += blockDim.x) a.csct[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
        char* p = (char*)st + kStepFieldsOffset;
        for (size_t i = 0; i < sizeof(DevState) - kStepFieldsOffset; ++i) p[i] = 0;
    }
}

// ------------------------------------------------------------------ K3 commit (+ finalize)
// k_resolve: one thread per full cell, tiles of kBlock full cells: its attempts whose
// claim holds the own ordinal won; writes the win mask, the mask of wins that go to
// the Border list, the tile's two win counts and adds them to its supertile.
// k_commit: winners are ranked per destination list in full-cell then direction
// order (tile prefix from the supertile and tile counts) and take recycled slots
// first, then appended slots, like omp_getNextFreeSlotInRXFront*(CELLRECYCLE); the
// full cell then becomes recrystallized (grid = ndefg + rxg, counts, slot INACTIVE).
__device__ __forceinline__ uint32_t commit_tiles(const DomainArgs& a) { return (full_cells(a) + kBlock - 1) / kBlock; }

template <bool ONE>
__global__ void __launch_bounds__(kBlock, 4) k_resolve(int base, int ndom) {
    __shared__ uint32_t s_pre[kMaxSegs + 1];
    __shared__ uint32_t s_a[kWarps], s_b[kWarps];
    const uint32_t total = ONE ? commit_tiles(c_args[base])
                               : seg_prefix(s_pre, ndom, [&](int s) { return commit_tiles(c_args[base + (s)]); });
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int s = ONE ? 0 : seg_find(s_pre, ndom, u);
        const DomainArgs& a = c_args[base + (s)];
        const uint32_t tile = ONE ? u : u - s_pre[s];
        const uint32_t F0 = a.st->nfull[0], F = F0 + a.st->nfull[1];
        const uint32_t f = tile * kBlock + threadIdx.x;
        uint32_t win = 0, tob = 0;
        if (f < F) {
            const uint32_t mask = a.amask[f];
            if (mask) {
                const int L = f >= F0 ? 1 : 0;
                const uint32_t cell = a.fcell[f];
                int x, y, z;
                decode(a, cell, x, y, z);
                const bool allB = (L == 0) && !(x > 1 && x < (int)a.nx - 2 && y > 1 && y < (int)a.ny - 2 && z > 1 && z < (int)a.nz - 2);
                uint32_t cl[26];
                uint32_t inter_m = 0;
#pragma unroll
                for (int d = 0; d < 26; ++d) {
                    cl[d] = kClaimFree;
                    if ((mask >> d) & 1u) {
                        uint32_t t;
                        bool inter;
                        target_of(a, L, x, y, z, d, t, inter);
                        cl[d] = a.claim[t];
                        if (inter) inter_m |= 1u << d;
                    }
                }
#pragma unroll
                for (int d = 0; d < 26; ++d) {
                    if (cl[d] == f * 26u + (uint32_t)d) {
                        win |= 1u << d;
                        // Inside full cells near a face infect into the Border list (:4606-4609);
                        // Border full cells send strictly interior targets to the Inside list (:4387)
                        if (L == 0 ? allB : !((inter_m >> d) & 1u)) tob |= 1u << d;
                    }
                }
            }
            a.amask[f] = win;
            a.tobm[f] = tob;
        }
        uint32_t cB = __popc(tob), cA = __popc(win) - cB;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) { cA += __shfl_down_sync(0xFFFFFFFFu, cA, o); cB += __shfl_down_sync(0xFFFFFFFFu, cB, o); }
        if (lane == 0) { s_a[warp] = cA; s_b[warp] = cB; }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t ta = 0, tb = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) { ta += s_a[w]; tb += s_b[w]; }
            a.ctcnt[2 * tile] = ta;
            a.ctcnt[2 * tile + 1] = tb;
            if (ta) atomicAdd(&a.csct[2 * (tile / kSuper)], ta);
            if (tb) atomicAdd(&a.csct[2 * (tile / kSuper) + 1], tb);
        }
        __syncthreads();
    }
}

// warp-reduced running P max (ordered bits of a positive double) and tagged-cell count
__device__ __forceinline__ void flush_new(const DomainArgs& a, double pmax, uint32_t ntag) {
    unsigned long long b = (unsigned long long)__double_as_longlong(pmax);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long x = __shfl_xor_sync(0xFFFFFFFFu, b, o);
        if (x > b) b = x;
        ntag += __shfl_xor_sync(0xFFFFFFFFu, ntag, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (b) atomicMax(&a.st->pmax_bits, b);
        if (ntag) atomicAdd(&a.st->ntagged, ntag);
    }
}

template <bool FP32, bool ONE>
__global__ void __launch_bounds__(kBlock, ONE ? 4 : 3) k_commit(int base, int ndom, uint32_t grow_tile) {
    __shared__ uint32_t s_pre[kMaxSegs + 1];
    __shared__ uint32_t s_a[kWarps], s_b[kWarps], s_w[kWarps], s_base[2];
    // per full cell of the tile: win masks, first ranks, cell (| Border list << 31), grain, overshoot
    __shared__ uint32_t s_off[kBlock + 1], s_win[kBlock], s_tob[kBlock], s_rA[kBlock], s_rB[kBlock], s_cell[kBlock], s_rsrc[kBlock];
    __shared__ double s_over[kBlock];
    const uint32_t total = ONE ? commit_tiles(c_args[base])
                               : seg_prefix(s_pre, ndom, [&](int s) { return commit_tiles(c_args[base + (s)]); });
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int cur = -1;           // domain whose P max and tag count are being accumulated
    double pmax = 0.0;      // max of the new positive weights
    uint32_t ntag = 0;      // new cells waiting for the host
    for (uint32_t u = blockIdx.x; u < total; u += gridDim.x) {
        const int s = ONE ? 0 : seg_find(s_pre, ndom, u);
        if (s != cur) {
            if (cur >= 0) flush_new(c_args[base + cur], pmax, ntag);
            cur = s; pmax = 0.0; ntag = 0;
        }
        const DomainArgs& a = c_args[base + (s)];
        const uint32_t tile = ONE ? u : u - s_pre[s];
        const uint32_t F0 = a.st->nfull[0], F = F0 + a.st->nfull[1];
        const uint32_t f = tile * kBlock + threadIdx.x;
        if (warp == 0) {
            uint32_t pa, pb;
            tile_prefix(a.ctcnt, a.csct, tile, pa, pb);
            if (lane == 0) { s_base[0] = pa; s_base[1] = pb; }
        }
        const uint32_t win = f < F ? a.amask[f] : 0u, tob = f < F ? a.tobm[f] : 0u;
        const uint32_t cB = __popc(tob), cA = __popc(win) - cB, cW = cA + cB;
        uint32_t iA = cA, iB = cB, iW = cW;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t xa = __shfl_up_sync(0xFFFFFFFFu, iA, o), xb = __shfl_up_sync(0xFFFFFFFFu, iB, o);
            const uint32_t xw = __shfl_up_sync(0xFFFFFFFFu, iW, o);
            if (lane >= o) { iA += xa; iB += xb; iW += xw; }
        }
        if (lane == 31) { s_a[warp] = iA; s_b[warp] = iB; s_w[warp] = iW; }
        // the full cell's own data, loaded while the scans complete
        const int L = f >= F0 ? 1 : 0;
        uint32_t slot = 0, cell = 0, rsrc = 0, gsrc = 0;
        double over = 0.0;  // the full cell's overshoot, for the cells it infects
        if (f < F) {
            slot = a.f[L].full[L ? f - F0 : f];
            cell = a.fcell[f];
            rsrc = a.f[L].rxg[slot];
            gsrc = a.f[L].defg[slot];
            if (win) {  // loaded with the grain ids, one round trip
                if (!FP32) over = __dsub_rn(((const double*)a.f[L].fill)[slot], 1.0);
                else over = (double)((((const float*)a.f[L].fill)[slot] - 1.0f) - a.f[L].comp[slot]);
            }
        }
        __syncthreads();
        uint32_t rA = s_base[0] + iA - cA, rB = s_base[1] + iB - cB, oW = iW - cW;
#pragma unroll
        for (int w = 0; w < kWarps; ++w)
            if (w < warp) { rA += s_a[w]; rB += s_b[w]; oW += s_w[w]; }
        if (threadIdx.x == 0 && tile + 1 == (ONE ? total : s_pre[s + 1] - s_pre[s])) {  // the domain's last tile: totals
            uint32_t ta = 0, tb = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) { ta += s_a[w]; tb += s_b[w]; }
            a.st->nwin[0] = s_base[0] + ta;
            a.st->nwin[1] = s_base[1] + tb;
        }
        s_off[threadIdx.x] = oW;
        if (threadIdx.x == kBlock - 1) s_off[kBlock] = oW + cW;
        s_win[threadIdx.x] = win;
        s_tob[threadIdx.x] = tob;
        s_rA[threadIdx.x] = rA;
        s_rB[threadIdx.x] = rB;
        s_cell[threadIdx.x] = cell | ((uint32_t)L << 31);
        s_rsrc[threadIdx.x] = rsrc;
        if (win) s_over[threadIdx.x] = over;
        __syncthreads();
        // every win of the tile by all threads: win k belongs to the full cell t with
        // s_off[t] <= k < s_off[t + 1]; its direction is the (k - s_off[t])-th set bit and
        // its rank in the destination list counts the cell's earlier wins there
        const uint32_t W = s_off[kBlock];
        for (uint32_t k = threadIdx.x; k < W; k += kBlock) {
            int lo = 0, hi = kBlock - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_off[mid] <= k) lo = mid;
                else hi = mid - 1;
            }
            const int t = lo;
            const uint32_t m = s_win[t], tb = s_tob[t];
            const int d = (int)__fns(m, 0u, (int)(k - s_off[t]) + 1);
            const int D = (tb >> d) & 1u;
            const uint32_t below = m & ((1u << d) - 1u);
            const uint32_t r = D ? s_rB[t] + __popc(below & tb) : s_rA[t] + __popc(below & ~tb);
            const uint32_t sc = s_cell[t];
            const int Ls = (int)(sc >> 31);
            int x, y, z;
            decode(a, sc & 0x7FFFFFFFu, x, y, z);
            uint32_t tgt;
            bool inter;
            target_of(a, Ls, x, y, z, d, tgt, inter);
            const uint32_t gt = a.grid[tgt];  // in flight together with the slot's load
            const DFront& dst = a.f[D];
            const uint32_t nrec = a.st->nrec[D];
            const uint32_t ns = r < nrec ? dst.recyc[r] : a.st->next_never[D] + (r - nrec);
            if (ns >= dst.cap) { atomicOr(&a.st->err, kErrCapacity); continue; }
            if (D == 1 && a.border_policy == 0 && r >= nrec && ns >= a.border_ref_cap) atomicOr(&a.st->err, kErrBorderRef);
            const double pf = a.pforce[gt];  // in flight together with the weight's load
            const int cls = c_cls[d];
            if (!FP32) {
                const double fac = cls == 1 ? 0.0682 : (cls == 2 ? 0.0542 : 0.0484);
                ((double*)dst.fill)[ns] = __dmul_rn(s_over[t], fac);
            } else {
                const float fac = cls == 1 ? 0.0682f : (cls == 2 ? 0.0542f : 0.0484f);
                ((float*)dst.fill)[ns] = (float)s_over[t] * fac;
                dst.comp[ns] = 0.0f;
            }
            const uint32_t rs = s_rsrc[t];
            dst.defg[ns] = gt;
            dst.rxg[ns] = rs;
            dst.xyz[ns] = tgt;
            a.grid[tgt] = 4096002000u;  // CURRENTLY_INFECTED
            a.claim[tgt] = kClaimFree;
            // mobility weight and cached velocity factor of the new cell
            double P = 0.0;
            uint32_t tag = 0;
            if (lookup_p(a, rs, gt, P, tag)) {
                const double mo = mobility(a, P);
                dst.mob[ns] = mo;
                const double v = velocity_from_force(mo, pf, c_code[d]);
                if (!FP32) {
                    // the increment with this step's dt: valid next step unless dt changes, when
                    // k_grow_fill recomputes every increment from vel anyway
                    ((double*)dst.vel)[ns] = v;
                    dst.inc[ns] = __double_as_longlong(v) >= 0 ? __dmul_rn(__dmul_rn(v, a.dt), a.cinv) : v;
                } else {
                    ((float*)dst.vel)[ns] = (float)v;
                }
                dst.dir[ns] = c_code[d];
                if (P > pmax) pmax = P;
            } else {
                // vel holds the answer tag until the next k_grow_fill
                if (!FP32) ((unsigned long long*)dst.vel)[ns] = tag;
                else ((uint32_t*)dst.vel)[ns] = tag;
                dst.dir[ns] = c_code[d] | kStale | kPend;
                ++ntag;
            }
        }
        if (f < F) {
            // the full cell is now recrystallized
            const DFront& src = a.f[L];
            a.grid[cell] = a.ndefg + rsrc;
            src.dir[slot] = kInactive;
            if (!FP32) ((double*)src.fill)[slot] = 0.0;
            else { ((float*)src.fill)[slot] = 0.0f; src.comp[slot] = 0.0f; }
        }
        // per-grain cell counts: one atomic per grain and warp (full cells of one grain
        // tend to finish together)
        {
            const bool has = f < F;
            const uint32_t act = __ballot_sync(0xFFFFFFFFu, has);
            const uint32_t mr = __match_any_sync(0xFFFFFFFFu, has ? rsrc : 0xFFFFFFFFu) & act;
            const uint32_t mg = __match_any_sync(0xFFFFFFFFu, has ? gsrc : 0xFFFFFFFFu) & act;
            if (has && (__ffs(mr) - 1) == lane) atomicAdd(&a.rxg_cnt[rsrc], (uint32_t)__popc(mr));
            if (has && (__ffs(mg) - 1) == lane) {
                const uint32_t k = (uint32_t)__popc(mg);
                const uint32_t old = atomicSub(&a.defg_cnt[gsrc], k);
                if (old == k) {
                    const uint32_t q = atomicAdd(&a.st->ndepleted, 1u);
                    if (q < a.ndefg) a.depleted[q] = gsrc;
                }
            }
        }
        __syncthreads();
    }
    if (cur >= 0) flush_new(c_args[base + cur], pmax, ntag);
    if (ONE) {
        // a single domain's step ends in the last block to finish (no separate launch)
        const DomainArgs& a = c_args[base];
        if (!a.active) return;
        __shared__ bool s_last;
        // the block's stores before its count: the barrier orders them before thread 0's fence, which
        // is cumulative (one fence per block instead of one per thread)
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            s_last = atomicAdd(&a.st->commit_done, 1u) == gridDim.x - 1;
        }
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        step_end_block(a, grow_tile);
    }
}

// One block per domain (batches; a single domain closes its step in the commit's last block).
__global__ void __launch_bounds__(kBlock) k_step_end(int base, int ndom, uint32_t grow_tile) {
    const DomainArgs& a = c_args[base + (blockIdx.x)];
    if (!a.active) return;
    step_end_block(a, grow_tile);
}

}  // namespace score
