// pp_host.h -- small helpers shared by the C ABI implementation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pp_host {

// dst[slot] = src[id_of_slot[slot]] for float arrays (device memory)
void gather_f32_sorted(const float* src_by_id, const uint32_t* id_of_slot, uint64_t n, float* dst, cudaStream_t s);
// dst[i] = v (device memory)
void fill_f32(float* dst, uint64_t n, float v, cudaStream_t s);
// Fisher-Yates over a copy of `label` driven by splitmix64(seed) (host memory)
void shuffle_labels(const uint8_t* label, uint64_t n, uint64_t seed, uint8_t* out);

}  // namespace pp_host
