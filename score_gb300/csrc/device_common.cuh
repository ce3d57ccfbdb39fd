// Device-side building blocks shared by the growth kernels: launch constants, error
// flags, the per-domain device scalars and the direction tables of the Moore stencil
// in the reference's infection order.
#pragma once
#include <cstdint>

namespace score {

constexpr int kBlock = 256;                 // threads per block of the tiled kernels
constexpr int kWarps = kBlock / 32;
constexpr uint8_t kInactive = 0xFF;         // dir byte of an INACTIVE slot
constexpr uint8_t kStale = 0x40;            // dir bit: cached fill increment not computed yet
constexpr uint8_t kCodeMask = 0x3F;         // dir bits holding the infector code 0..26
constexpr uint32_t kClaimFree = 0xFFFFFFFFu;
constexpr uint8_t kPend = 0x80;             // dir bit: vel holds an answer tag, P comes from the host
constexpr unsigned long long kPtabEmpty = 0xFFFFFFFFFFFFFFFFull;    // NaN bit pattern, never a weight
constexpr unsigned long long kPtabTag = 0xFFFE000000000000ull;      // | m: requested from the host as miss m
constexpr unsigned long long kMissVoid = 0xFFFFFFFFFFFFFFFFull;     // miss slot lost a race: no request

// error flags (DevState::err)
constexpr uint32_t kErrTimeout = 1u << 0;    // kept for the status code; no kernel waits on another
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
    uint32_t reserved[4];
    // ---- per step ----
    uint32_t nfull[2];          // FullRX list lengths
    uint32_t ninactive[2];      // INACTIVE slots seen by the scan (uncapped)
    uint32_t nrec[2];           // recycle list lengths = min(ninactive, cap)
    uint32_t nwin[2];           // newly infected cells per destination list
    uint32_t nmiss;             // (rxg,defg) pairs whose P the host must compute
    uint32_t ntagged;           // new cells whose P waits for the host (tagged)
    uint32_t ndepleted;         // deformed grains whose last cell recrystallized
    uint32_t nnuc;              // nuclei placed on the device before this step's grow
    uint32_t commit_done;       // commit blocks finished (the last one closes the step)
    unsigned long long sv[2];   // ACTIVE slots updated
    unsigned long long pmax_bits;  // max over new non-negative P (ordered bits)
    double dv[2];               // sum of fill increments
};
constexpr size_t kStepFieldsOffset = 32;  // offsetof(DevState, nfull)

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Moore stencil in the order the reference issues infections
// (updateFullRXInside, SCORE_Kernel.cpp:4611-4638): offsets, direction code
// stored as the new cell's infector, and overshoot class (1 face, 2 edge, 3 corner).
#define SCORE_STENCIL_DX {-1, 0, 1, -1, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1, -1, 0, 1}
#define SCORE_STENCIL_DY {-1, -1, -1, 0, 0, 1, 1, 1, 1, 1, 1, -1, -1, -1, 0, 0, 0, -1, -1, -1, 0, 0, 0, 1, 1, 1}
#define SCORE_STENCIL_DZ {0, 0, 0, 0, 0, 0, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, 1}
__constant__ int8_t c_dx[26] = SCORE_STENCIL_DX;
__constant__ int8_t c_dy[26] = SCORE_STENCIL_DY;
__constant__ int8_t c_dz[26] = SCORE_STENCIL_DZ;
// the same offsets for host code (linear neighbour offsets of interior cells)
constexpr int8_t kStencilDx[26] = SCORE_STENCIL_DX;
constexpr int8_t kStencilDy[26] = SCORE_STENCIL_DY;
constexpr int8_t kStencilDz[26] = SCORE_STENCIL_DZ;
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
