// Percolation analysis of a domain's recrystallized and infected cells on the device (percolation.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include "../../include/score_gb300.h"

namespace score {

// Clusters of the cells whose grid value is >= ndefg, over the device grid `grid` (nx x ny x nz, x
// fastest): count, largest, spanning axes, ascending sizes (up to sizes_cap) and, if `labels` is not
// null, every cell's compact label (host buffer, N values).  mode SCORE_PERC_*.
int percolation_analyze(const uint32_t* grid, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t ndefg, int mode, cudaStream_t st,
                        int sms, score_perc_result* out, uint32_t* sizes, uint32_t sizes_cap, uint32_t* labels, std::string& err);

}  // namespace score
