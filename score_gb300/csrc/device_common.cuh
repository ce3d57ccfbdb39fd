// Device-side building blocks shared by the growth kernels: direction tables of
// the Moore stencil in the reference's infection order, relaxed/acquire memory
// accessors, and the decoupled look-back tile scan used for every ordered
// stream compaction (FullRX list, recycle list, new-cell slot ranks).
#pragma once
#include <cstdint>

namespace score {

constexpr int kBlock = 256;                 // threads per block of the tiled kernels
constexpr int kWarps = kBlock / 32;
constexpr uint8_t kInactive = 0xFF;         // dir byte of an INACTIVE slot
constexpr uint8_t kStale = 0x40;            // dir bit: cached fill increment not computed yet
constexpr uint8_t kCodeMask = 0x3F;         // dir bits holding the infector code 0..26
constexpr uint32_t kClaimFree = 0xFFFFFFFFu;
constexpr unsigned long long kPtabEmpty = 0xFFFFFFFFFFFFFFFFull;    // NaN bit pattern, never a weight
constexpr unsigned long long kPtabPending = 0xFFFFFFFFFFFFFFFEull;  // requested from the host this step
constexpr uint32_t kSpinLimit = 1u << 22;   // bounded waits: give up, flag, return

// error flags (DevState::err)
constexpr uint32_t kErrTimeout = 1u << 0;
constexpr uint32_t kErrCapacity = 1u << 1;
constexpr uint32_t kErrBorderRef = 1u << 2;
constexpr uint32_t kErrKeyLimit = 1u << 3;
constexpr uint32_t kErrBounds = 1u << 4;
constexpr uint32_t kErrMissCap = 1u << 5;

// Per-domain device scalars.  The fields from `nfull` on are zeroed at the start of
// every step (one memset of the tail of the struct); next_never and err persist.
struct DevState {
    uint32_t next_never[2];     // slots ever used per list (Inside, Border)
    uint32_t err;               // sticky error flags
    uint32_t err_info;
    uint32_t tiles_used[3];     // look-back tiles the last grow (x2) and commit launches used
    uint32_t pad0;
    // ---- per step ----
    uint32_t nfull[2];          // FullRX list lengths
    uint32_t ninactive[2];      // INACTIVE slots seen by the scan (uncapped)
    uint32_t nrec[2];           // recycle list lengths = min(ninactive, cap)
    uint32_t nwin[2];           // newly infected cells per destination list
    uint32_t nmiss;             // (rxg,defg) pairs whose P the host must compute
    uint32_t npending;          // new cells whose P waits for the host
    uint32_t ndepleted;         // deformed grains whose last cell recrystallized
    uint32_t pad;
    unsigned long long sv[2];   // ACTIVE slots updated
    unsigned long long pmax_bits;  // max over new non-negative P (ordered bits)
    double dv[2];               // sum of fill increments
};
constexpr size_t kStepFieldsOffset = 32;  // offsetof(DevState, nfull)

// ---- memory order helpers (device scope) ----
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- decoupled look-back over tiles carrying two 31-bit counters ----
// status word: bit 63 = inclusive prefix ready, bit 62 = tile aggregate ready,
// bits 61..31 counter A, bits 30..0 counter B.
constexpr unsigned long long kFlagIncl = 1ull << 63;
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kMask31 = 0x7FFFFFFFull;
__device__ __forceinline__ unsigned long long pack2(uint32_t a, uint32_t b) {
    return ((unsigned long long)(a & kMask31) << 31) | (unsigned long long)(b & kMask31);
}

// Called by ALL 32 lanes of one warp of the block owning `tile` (warp-parallel
// look-back: each round inspects 32 predecessors at once).  Returns, in every lane,
// the exclusive prefix of both counters over all earlier tiles and publishes this
// tile's inclusive prefix.  Waits are bounded: after kSpinLimit polls the error flag
// is set and the partial sum is used (results are then invalid and the host reports
// SCORE_ERR_TIMEOUT).
__device__ __forceinline__ void lookback2(unsigned long long* status, uint32_t tile, uint32_t aggA, uint32_t aggB,
                                          uint32_t& exA, uint32_t& exB, uint32_t* err) {
    const int lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) st_release_u64(&status[0], kFlagIncl | pack2(aggA, aggB));
        exA = 0; exB = 0;
        return;
    }
    if (lane == 0) st_release_u64(&status[tile], kFlagAgg | pack2(aggA, aggB));
    uint32_t accA = 0, accB = 0;
    int64_t j = (int64_t)tile - 1;
    bool timed_out = false;
    while (j >= 0) {
        const int64_t idx = j - lane;  // lane 0 looks at the nearest predecessor
        unsigned long long s = kFlagIncl;  // before tile 0: an inclusive zero
        if (idx >= 0) {
            uint32_t polls = 0;
            for (;;) {
                s = ld_acquire_u64(&status[idx]);
                if (s & (kFlagIncl | kFlagAgg)) break;
                if (++polls > kSpinLimit) { timed_out = true; s = kFlagIncl; break; }
                if (polls > 32) __nanosleep(32);
            }
        }
        const uint32_t incl = __ballot_sync(0xFFFFFFFFu, (s & kFlagIncl) != 0);
        const int stop = incl ? __ffs(incl) - 1 : 31;  // nearest inclusive predecessor in this window
        uint32_t a = lane <= stop ? (uint32_t)((s >> 31) & kMask31) : 0u;
        uint32_t b = lane <= stop ? (uint32_t)(s & kMask31) : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
            b += __shfl_xor_sync(0xFFFFFFFFu, b, o);
        }
        accA += a; accB += b;
        if (incl) break;
        j -= 32;
    }
    if (__any_sync(0xFFFFFFFFu, timed_out) && lane == 0) atomicOr(err, kErrTimeout);
    if (lane == 0) st_release_u64(&status[tile], kFlagIncl | pack2(accA + aggA, accB + aggB));
    exA = accA; exB = accB;
}

// Moore stencil in the order the reference issues infections
// (updateFullRXInside, SCORE_Kernel.cpp:4611-4638): offsets, direction code
// stored as the new cell's infector, and overshoot class (1 face, 2 edge, 3 corner).
__constant__ int8_t c_dx[26] = {-1, 0, 1, -1, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1};
__constant__ int8_t c_dy[26] = {-1, -1, -1, 0, 0, 1, 1, 1, 1, 1, 1, -1, -1, -1, 0, 0, 0, -1, -1, -1, 0, 0, 0, 1, 1, 1};
__constant__ int8_t c_dz[26] = {0, 0, 0, 0, 0, 0, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
__constant__ uint8_t c_code[26] = {16, 15, 14, 13, 12, 11, 10, 9, 19, 18, 17, 25, 24, 23, 22, 21, 20, 8, 7, 6, 5, 4, 3, 2, 1, 0};
__constant__ uint8_t c_cls[26] = {2, 1, 2, 1, 1, 2, 1, 2, 3, 2, 3, 3, 2, 3, 2, 1, 2, 3, 2, 3, 2, 1, 2, 3, 2, 3};
// velocity shape factor indexed by infector code (calcGrowthStepInside, SCORE_Kernel.cpp:4053-4055); 26 = nucleus
__constant__ double c_sf[27] = {0.6494, 0.7957, 0.6494, 0.7957, 1.0000, 0.7957, 0.6494, 0.7957, 0.6494,
                                0.7957, 1.0000, 0.7957, 1.0000, 1.0000, 0.7957, 1.0000, 0.7957,
                                0.6494, 0.7957, 0.6494, 0.7957, 1.0000, 0.7957, 0.6494, 0.7957, 0.6494, 1.0};
__constant__ float c_sf32[27] = {0.6494f, 0.7957f, 0.6494f, 0.7957f, 1.0000f, 0.7957f, 0.6494f, 0.7957f, 0.6494f,
                                 0.7957f, 1.0000f, 0.7957f, 1.0000f, 1.0000f, 0.7957f, 1.0000f, 0.7957f,
                                 0.6494f, 0.7957f, 0.6494f, 0.7957f, 1.0000f, 0.7957f, 0.6494f, 0.7957f, 0.6494f, 1.0f};

}  // namespace score
