/*
 * scan.cuh -- exclusive prefix sum of u64 arrays in place on the device, in
 * blocks of 1,024 elements: k_scan_local scans each block and writes its
 * total, the block totals are scanned the same way (recursively, by the
 * caller), and k_scan_add adds each block's offset. Used by the level
 * builders of both search modes (child offsets and kept-child ranks), so
 * no level's counts make a round trip through host memory.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int kScanBlock = 1024;  /* elements per block (256 threads x 4) */

__global__ void k_scan_local(uint64_t *a, uint64_t n, uint64_t *block_sums)
{
    __shared__ uint64_t sh[256];
    const uint64_t base = (uint64_t)blockIdx.x * kScanBlock + threadIdx.x * 4;
    uint64_t v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = base + k < n ? a[base + k] : 0;
        s += v[k];
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        uint64_t x = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += x;
        __syncthreads();
    }
    uint64_t run = sh[threadIdx.x] - s;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (base + k < n) a[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 255) block_sums[blockIdx.x] = sh[255];
}

__global__ void k_scan_add(uint64_t *a, uint64_t n, const uint64_t *block_off)
{
    const uint64_t base = (uint64_t)blockIdx.x * kScanBlock;
    const uint64_t add = block_off[blockIdx.x];
    for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x)
        if (base + k < n) a[base + k] += add;
}

}  // namespace
