// sm_103a kernels of one recrystallization growth step.
//
//   k_grow      per list: FP64 (or FP32+Kahan) fill update of every ACTIVE slot in
//               [0, next_never), ordered compaction of full slots (FullRX list) and of
//               INACTIVE slots (recycle list, capped), fused Sv / dV reductions.
//               caregionMemHdl::ompshar_sim_myCA_calcGrowthStep{Inside,Border},
//               SCORE_Kernel.cpp:4046-4130, 4183-4249.
//   k_claim     one thread per infection attempt (full cell x 26 directions, in the
//               reference's sequential order = the attempt ordinal): atomicMin of the
//               ordinal into the target's claim word if the target is still deformed.
//   k_commit    winners (claim == own ordinal) are ranked per destination list in
//               ordinal order (look-back scan) and take recycled slots first, then
//               appended ones, exactly like omp_getNextFreeSlotInRXFront*(CELLRECYCLE);
//               the new front cell gets the overshoot carry, P, grain ids.
//               ompshar_sim_myCA_updateFullRX{Inside,Border} + omp_infect_OutOfRXFront*,
//               SCORE_Kernel.cpp:4252-4774.
//   k_finalize  full cells become recrystallized: grid label ndefg+rxg, grain counts,
//               slot INACTIVE (the tail of the same functions, :4640-4653, :4752-4764).
#pragma once
#include <cstdint>
#include "device_common.cuh"

namespace score {

struct DFront {
    void* fill;          // double (FP64) or float (FP32)
    float* comp;         // Kahan compensation (FP32 only)
    void* P;             // double (FP64) or float (FP32)
    uint32_t* defg;
    uint32_t* rxg;
    uint32_t* xyz;       // linear cell index x + y nx + z nx ny
    uint8_t* dir;        // infector code 0..26, kInactive = INACTIVE
    uint32_t* full;      // FullRX list (slot indices, slot order)
    uint32_t* recyc;     // recycle list (slot indices, slot order, capped)
    uint32_t cap;        // device capacity of the slot arrays
    uint32_t reccap;     // ntotalRecyclingList of the reference
};

struct DomainArgs {
    DFront f[2];
    DevState* st;
    uint32_t* grid;
    uint32_t* claim;
    unsigned long long* ptab;   // nrxg x ndefg mobility weights as bits (kPtabEmpty = unknown)
    const double* pforce;       // per deformed grain driving force (FP64)
    const float* pforce32;
    uint32_t* defg_cnt;
    uint32_t* rxg_cnt;
    uint32_t* depleted;
    unsigned long long* miss;   // table indices the host must fill
    uint32_t* pending;          // (list << 31) | slot of new cells waiting for P
    uint32_t misscap, pendcap;
    uint32_t nx, ny, nz, nxy;
    uint32_t ndefg, nrxg;
    uint32_t border_ref_cap;
    int32_t border_policy, boundary, mobility_model;
    double mLAGB, mHAGB, mGS, mRH, dt, cinv;
    float mLAGB32, mHAGB32, mGS32, mRH32, dtc32;
};

__device__ __forceinline__ void decode(const DomainArgs& a, uint32_t cell, int& x, int& y, int& z) {
    z = (int)(cell / a.nxy);
    uint32_t r = cell - (uint32_t)z * a.nxy;
    y = (int)(r / a.nx);
    x = (int)(r - (uint32_t)y * a.nx);
}

// Target cell of attempt d from a cell of list L.  Inside cells are strictly interior
// so their neighbours need no wrap; Border cells wrap x,y periodically and drop z
// (reference) or wrap z (periodic build option).  Returns false if the attempt is dropped.
__device__ __forceinline__ bool target_of(const DomainArgs& a, int L, uint32_t cell, int d, uint32_t& t) {
    int x, y, z;
    decode(a, cell, x, y, z);
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
    t = (uint32_t)tx + a.nx * ((uint32_t)ty + a.ny * (uint32_t)tz);
    return true;
}

// Inside full cells closer than 2 cells to a face send every infection to the Border
// list (InfectIntoBorder, SCORE_Kernel.cpp:4606-4609).
__device__ __forceinline__ bool into_border(const DomainArgs& a, uint32_t cell) {
    int x, y, z;
    decode(a, cell, x, y, z);
    return !(x > 1 && x < (int)a.nx - 2 && y > 1 && y < (int)a.ny - 2 && z > 1 && z < (int)a.nz - 2);
}
// Border full cells route strictly interior targets to the Inside list (:4387).
__device__ __forceinline__ bool strictly_interior(const DomainArgs& a, uint32_t cell) {
    int x, y, z;
    decode(a, cell, x, y, z);
    return x > 0 && x < (int)a.nx - 1 && y > 0 && y < (int)a.ny - 1 && z > 0 && z < (int)a.nz - 1;
}

// warp-0 exclusive scan of 2*32 tile counters laid out [item][warp]; returns the two
// tile totals in lane 0.  cntA/cntB are rewritten with exclusive offsets.
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

// ------------------------------------------------------------------ K1 grow
template <bool FP32>
__global__ void __launch_bounds__(kBlock) k_grow(DomainArgs a, int L, unsigned long long* status, uint32_t* ticket) {
    constexpr int ITEMS = 8;  // ITEMS * kWarps must be 64 for scan64_pair
    constexpr uint32_t TILE = kBlock * ITEMS;
    const DFront fr = a.f[L];
    const uint32_t n = a.st->next_never[L];
    const uint32_t ntiles = (n + TILE - 1) / TILE;
    __shared__ uint32_t s_tile, s_exF, s_exI;
    __shared__ uint32_t s_cntF[ITEMS * kWarps], s_cntI[ITEMS * kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long sv = 0;
    double dv = 0.0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t base = tile * TILE;
        uint32_t fm[ITEMS], im[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t slot = base + (uint32_t)(k * kBlock) + threadIdx.x;
            const bool valid = slot < n;
            const uint8_t d = valid ? fr.dir[slot] : kInactive;
            const bool inact = valid && d == kInactive;
            bool full = false;
            if (valid && d != kInactive) {
                ++sv;
                const uint32_t g = fr.defg[slot];
                if (!FP32) {
                    const double P = ((const double*)fr.P)[slot];
                    double m;
                    if (a.mobility_model == 2) m = __dmul_rn(P, a.mRH);
                    else if (P < 0.0) m = a.mLAGB;
                    else m = __dadd_rn(__dmul_rn(P, a.mGS), __dmul_rn(__dsub_rn(1.0, P), a.mHAGB));
                    const double p = a.pforce[g];
                    if (p > 5.0e-16) {
                        double v = __dmul_rn(m, p);
                        v = __dmul_rn(v, c_sf[d]);
                        const double inc = __dmul_rn(__dmul_rn(v, a.dt), a.cinv);
                        const double f = __dadd_rn(((double*)fr.fill)[slot], inc);
                        ((double*)fr.fill)[slot] = f;
                        dv += inc;
                        full = f >= 1.0;
                    }
                } else {
                    const float P = ((const float*)fr.P)[slot];
                    float m;
                    if (a.mobility_model == 2) m = P * a.mRH32;
                    else if (P < 0.0f) m = a.mLAGB32;
                    else m = P * a.mGS32 + (1.0f - P) * a.mHAGB32;
                    const float p = a.pforce32[g];
                    if (p > 5.0e-16f) {
                        const float inc = m * p * c_sf32[d] * a.dtc32;
                        // Kahan-compensated accumulation of the fill
                        const float f0 = ((float*)fr.fill)[slot];
                        const float y = inc - fr.comp[slot];
                        const float t = f0 + y;
                        const float cnew = (t - f0) - y;
                        fr.comp[slot] = cnew;
                        ((float*)fr.fill)[slot] = t;
                        dv += (double)inc;
                        full = (t - cnew) >= 1.0f;
                    }
                }
            }
            fm[k] = __ballot_sync(0xFFFFFFFFu, full);
            im[k] = __ballot_sync(0xFFFFFFFFu, inact);
            if (lane == 0) {
                s_cntF[k * kWarps + warp] = __popc(fm[k]);
                s_cntI[k * kWarps + warp] = __popc(im[k]);
            }
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t totF, totI;
            scan64_pair(s_cntF, s_cntI, totF, totI);
            if (lane == 0) {
                uint32_t exF, exI;
                lookback2(status, tile, totF, totI, exF, exI, &a.st->err);
                s_exF = exF; s_exI = exI;
                if (tile == ntiles - 1) {
                    a.st->nfull[L] = exF + totF;
                    a.st->ninactive[L] = exI + totI;
                    a.st->nrec[L] = min(exI + totI, fr.reccap);
                }
            }
        }
        __syncthreads();
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t slot = base + (uint32_t)(k * kBlock) + threadIdx.x;
            if ((fm[k] >> lane) & 1u) fr.full[s_exF + s_cntF[k * kWarps + warp] + __popc(fm[k] & lt)] = slot;
            if ((im[k] >> lane) & 1u) {
                const uint32_t r = s_exI + s_cntI[k * kWarps + warp] + __popc(im[k] & lt);
                if (r < fr.reccap) fr.recyc[r] = slot;
            }
        }
        __syncthreads();
    }
    // block-level reductions of the observation counters
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sv += __shfl_down_sync(0xFFFFFFFFu, sv, o);
        dv += __shfl_down_sync(0xFFFFFFFFu, dv, o);
    }
    if (lane == 0 && sv) {
        atomicAdd(&a.st->sv[L], sv);
        atomicAdd(&a.st->dv[L], dv);
    }
}

// ------------------------------------------------------------------ K2 claim
__device__ __forceinline__ bool attempt_total(const DomainArgs& a, uint32_t& F0, uint32_t& total) {
    F0 = a.st->nfull[0];
    const unsigned long long t = 26ull * ((unsigned long long)F0 + a.st->nfull[1]);
    if (t >= 0xFFFFFFFFull) return false;
    total = (uint32_t)t;
    return true;
}

__global__ void __launch_bounds__(kBlock) k_claim(DomainArgs a) {
    uint32_t F0, total;
    if (!attempt_total(a, F0, total)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.st->err, kErrKeyLimit);
        return;
    }
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < total; o += gridDim.x * blockDim.x) {
        const uint32_t f = o / 26u;
        const int d = (int)(o - f * 26u);
        const int L = f >= F0 ? 1 : 0;
        const uint32_t slot = a.f[L].full[L ? f - F0 : f];
        uint32_t t;
        if (!target_of(a, L, a.f[L].xyz[slot], d, t)) continue;
        if (a.grid[t] < a.ndefg) atomicMin(&a.claim[t], o);
    }
}

// P of a new cell: the infector's P when the deformed grain is the same, else the
// table entry; unknown entries are requested from the host (returned as pending).
__device__ __forceinline__ bool lookup_p(const DomainArgs& a, uint32_t rxg, uint32_t defg, double& P) {
    unsigned long long* e = &a.ptab[(unsigned long long)rxg * a.ndefg + defg];
    unsigned long long bits = *(volatile unsigned long long*)e;
    if (bits == kPtabEmpty) {
        unsigned long long old = atomicCAS(e, kPtabEmpty, kPtabPending);
        if (old == kPtabEmpty) {
            const uint32_t m = atomicAdd(&a.st->nmiss, 1u);
            if (m < a.misscap) a.miss[m] = (unsigned long long)rxg * a.ndefg + defg;
            else atomicOr(&a.st->err, kErrMissCap);
            return false;
        }
        bits = old;
    }
    if (bits == kPtabPending) return false;
    P = __longlong_as_double((long long)bits);
    return true;
}

// ------------------------------------------------------------------ K3 commit
template <bool FP32>
__global__ void __launch_bounds__(kBlock) k_commit(DomainArgs a, unsigned long long* status, uint32_t* ticket) {
    constexpr int ITEMS = 8;
    constexpr uint32_t TILE = kBlock * ITEMS;
    uint32_t F0, total;
    if (!attempt_total(a, F0, total)) return;
    const uint32_t ntiles = (total + TILE - 1) / TILE;
    __shared__ uint32_t s_tile, s_exA, s_exB;
    __shared__ uint32_t s_cntA[ITEMS * kWarps], s_cntB[ITEMS * kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t base = tile * TILE;
        uint32_t am[ITEMS], bm[ITEMS], tgt[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const uint32_t o = base + (uint32_t)(k * kBlock) + threadIdx.x;
            bool winA = false, winB = false;
            tgt[k] = 0;
            if (o < total) {
                const uint32_t f = o / 26u;
                const int d = (int)(o - f * 26u);
                const int L = f >= F0 ? 1 : 0;
                const uint32_t slot = a.f[L].full[L ? f - F0 : f];
                const uint32_t cell = a.f[L].xyz[slot];
                uint32_t t;
                if (target_of(a, L, cell, d, t) && a.claim[t] == o) {
                    const bool toBorder = (L == 0) ? into_border(a, cell) : !strictly_interior(a, t);
                    winA = !toBorder; winB = toBorder;
                    tgt[k] = t;
                }
            }
            am[k] = __ballot_sync(0xFFFFFFFFu, winA);
            bm[k] = __ballot_sync(0xFFFFFFFFu, winB);
            if (lane == 0) {
                s_cntA[k * kWarps + warp] = __popc(am[k]);
                s_cntB[k * kWarps + warp] = __popc(bm[k]);
            }
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t totA, totB;
            scan64_pair(s_cntA, s_cntB, totA, totB);
            if (lane == 0) {
                uint32_t exA, exB;
                lookback2(status, tile, totA, totB, exA, exB, &a.st->err);
                s_exA = exA; s_exB = exB;
                if (tile == ntiles - 1) { a.st->nwin[0] = exA + totA; a.st->nwin[1] = exB + totB; }
            }
        }
        __syncthreads();
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const bool wA = (am[k] >> lane) & 1u, wB = (bm[k] >> lane) & 1u;
            if (!(wA || wB)) continue;
            const int D = wB ? 1 : 0;
            const uint32_t r = wB ? s_exB + s_cntB[k * kWarps + warp] + __popc(bm[k] & lt)
                                  : s_exA + s_cntA[k * kWarps + warp] + __popc(am[k] & lt);
            const uint32_t o = base + (uint32_t)(k * kBlock) + threadIdx.x;
            const uint32_t f = o / 26u;
            const int d = (int)(o - f * 26u);
            const int L = f >= F0 ? 1 : 0;
            const uint32_t src = a.f[L].full[L ? f - F0 : f];
            const uint32_t t = tgt[k];
            const DFront& dst = a.f[D];
            const uint32_t nrec = a.st->nrec[D];
            const uint32_t ns = r < nrec ? dst.recyc[r] : a.st->next_never[D] + (r - nrec);
            if (ns >= dst.cap) { atomicOr(&a.st->err, kErrCapacity); continue; }
            if (D == 1 && a.border_policy == 0 && r >= nrec && ns >= a.border_ref_cap) atomicOr(&a.st->err, kErrBorderRef);
            const uint32_t gt = a.grid[t];
            const uint32_t gsrc = a.f[L].defg[src];
            const uint32_t rsrc = a.f[L].rxg[src];
            const int cls = c_cls[d];
            double P = 0.0;
            bool known = true;
            if (!FP32) {
                const double over = __dsub_rn(((const double*)a.f[L].fill)[src], 1.0);
                const double fac = cls == 1 ? 0.0682 : (cls == 2 ? 0.0542 : 0.0484);
                ((double*)dst.fill)[ns] = __dmul_rn(over, fac);
                if (gsrc == gt) P = ((const double*)a.f[L].P)[src];
                else known = lookup_p(a, rsrc, gt, P);
                ((double*)dst.P)[ns] = known ? P : __longlong_as_double((long long)kPtabEmpty);
            } else {
                const float over = (((const float*)a.f[L].fill)[src] - 1.0f) - a.f[L].comp[src];
                const float fac = cls == 1 ? 0.0682f : (cls == 2 ? 0.0542f : 0.0484f);
                ((float*)dst.fill)[ns] = over * fac;
                dst.comp[ns] = 0.0f;
                float P32 = 0.0f;
                if (gsrc == gt) { P32 = ((const float*)a.f[L].P)[src]; P = (double)P32; }
                else { known = lookup_p(a, rsrc, gt, P); P32 = (float)P; }
                ((float*)dst.P)[ns] = known ? P32 : __int_as_float(0x7FFFFFFF);
            }
            dst.dir[ns] = c_code[d];
            dst.defg[ns] = gt;
            dst.rxg[ns] = rsrc;
            dst.xyz[ns] = t;
            a.grid[t] = 4096002000u;  // CURRENTLY_INFECTED
            a.claim[t] = kClaimFree;
            if (!known) {
                const uint32_t q = atomicAdd(&a.st->npending, 1u);
                if (q < a.pendcap) a.pending[q] = ((uint32_t)D << 31) | ns;
                else atomicOr(&a.st->err, kErrMissCap);
            } else if (P > 0.0) {
                atomicMax(&a.st->pmax_bits, (unsigned long long)__double_as_longlong(P));
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ K4 finalize
template <bool FP32>
__global__ void __launch_bounds__(kBlock) k_finalize(DomainArgs a) {
    const uint32_t F0 = a.st->nfull[0], F = F0 + a.st->nfull[1];
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < F; f += gridDim.x * blockDim.x) {
        const int L = f >= F0 ? 1 : 0;
        const DFront& fr = a.f[L];
        const uint32_t slot = fr.full[L ? f - F0 : f];
        const uint32_t r = fr.rxg[slot], g = fr.defg[slot];
        a.grid[fr.xyz[slot]] = a.ndefg + r;
        atomicAdd(&a.rxg_cnt[r], 1u);
        const uint32_t old = atomicSub(&a.defg_cnt[g], 1u);
        if (old == 1u) {
            const uint32_t q = atomicAdd(&a.st->ndepleted, 1u);
            if (q < a.ndefg) a.depleted[q] = g;
        }
        fr.dir[slot] = kInactive;
        if (!FP32) ((double*)fr.fill)[slot] = 0.0;
        else { ((float*)fr.fill)[slot] = 0.0f; fr.comp[slot] = 0.0f; }
    }
}

// ------------------------------------------------------------------ K5 step end
__global__ void k_step_end(DevState* st, uint32_t cap0, uint32_t cap1) {
    const uint32_t cap[2] = {cap0, cap1};
    for (int D = 0; D < 2; ++D) {
        if (st->nwin[D] > st->nrec[D]) st->next_never[D] += st->nwin[D] - st->nrec[D];
        if (st->next_never[D] > cap[D]) { st->next_never[D] = cap[D]; st->err |= kErrCapacity; }
    }
}

}  // namespace score
