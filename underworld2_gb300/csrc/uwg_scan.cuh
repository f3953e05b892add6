// Device-wide exclusive prefix sum of int32 arrays (in place allowed):
// per-block warp-shuffle scan, recursive scan of the block totals, add-back.
#pragma once
#include "uwg_internal.cuh"

__global__ void k_scan_block(int64_t n, const int32_t* in, int32_t* out, int32_t* bsum);
__global__ void k_scan_add(int64_t n, int32_t* out, const int32_t* boff);

int uwg_scan_exclusive(uwg_ctx* c, const int32_t* in, int32_t* out, int64_t n);
