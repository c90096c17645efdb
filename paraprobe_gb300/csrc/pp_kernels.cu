// pp_kernels.cu -- sm_103a kernels of the GB300 spatial-statistics path.
//
//  K0 k_decode_pos     big-endian POS records -> xyz + ranged type ids
//  K1 k_cell_count / k_scan_* / k_scatter
//                      uniform-grid counting sort: ions -> cell-sorted float4
//                      records (x-fastest cells, so stencil rows are contiguous)
//  K2 k_surface_cells  squared ion-to-hull distance, same candidate test and
//                      float evaluation order as the reference
//  K3 k_scan<KR,EMAX>  warp-per-centre scan of the trimmed cell stencil: RDF
//                      bins in shared memory, kNN as register-resident sorted
//                      lists, neighbour counts; or pair-list count / emit
//  K5 k_apply          batched realisations over stored per-centre pair lists
//
// Floating-point rules.  Every quantity that decides a count is evaluated with
// round-to-nearest intrinsics in the reference's source order and without
// contraction (the library is built with --fmad=false as well):
//   d^2 = ((xi-xj)^2 + (yi-yj)^2) + (zi-zj)^2   src/PARAPROBE_KDTree.h:55-58
// Histogram bins are found by comparing d^2 with a host-built threshold table
// (the smallest float d^2 of each category under histogram::add,
// src/PARAPROBE_Histogram.h:97-117), so no double arithmetic runs per pair.

#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

#include "pp_internal.h"
#include "pp_host.h"
#include "../../include/paraprobe_gb300.h"

namespace pp {

#define FULL 0xffffffffu

// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `smem` bytes.  The limit only ever grows (per device and kernel, under
// a lock): serving threads launch the same kernels concurrently with
// different sizes, and lowering the limit between another thread's set-up and
// its launch would make that launch fail.
static bool allow_dynamic_smem(const void* fn, size_t smem) {
  if (smem <= 48 * 1024) return true;
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> granted;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lock(mu);
  size_t& g = granted[{dev, fn}];
  if (smem <= g) return true;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return false;
  g = smem;
  return true;
}

__device__ __forceinline__ float kInf() { return __int_as_float(0x7f800000); }

__device__ __forceinline__ float dist2(float ax, float ay, float az, float bx, float by, float bz) {
  const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Two floats in one 64-bit register pair, for the packed f32x2 arithmetic of
// sm_100+ (one instruction, two IEEE round-to-nearest results).
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// dist2 of one centre (its coordinates duplicated in each pair: cxx = (cx, cx)
// ...) against two ions whose x, y and z come as pairs: differences and
// squares packed, the two sums scalar, in dist2's order.  Bit-identical to
// dist2 on the GPU (checked on 2M random pairs); with the sums packed as well
// (add.rn.f32x2) the results differ from dist2 by an ulp or two for about one
// pair in five (measured on 134M pairs, with or without --fmad=false passed to
// ptxas: a product feeding only a packed add comes out unrounded, as from a
// fused multiply-add), so they are not.
__device__ __forceinline__ void dist2_x2(unsigned long long cxx, unsigned long long cyy, unsigned long long czz,
                                         unsigned long long xx, unsigned long long yy, unsigned long long zz,
                                         float& d0, float& d1) {
  const unsigned long long dx = f2_sub(cxx, xx), dy = f2_sub(cyy, yy), dz = f2_sub(czz, zz);
  float x0, x1, y0, y1, z0, z1;
  f2_unpack(f2_mul(dx, dx), x0, x1);
  f2_unpack(f2_mul(dy, dy), y0, y1);
  f2_unpack(f2_mul(dz, dz), z0, z1);
  d0 = __fadd_rn(__fadd_rn(x0, y0), z0);
  d1 = __fadd_rn(__fadd_rn(x1, y1), z1);
}

// ------------------------------------------------------------------ K0 / bbox
__device__ __forceinline__ uint32_t f2o(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// d_minmax holds 6 order-preserving keys (min x,y,z as min keys, max x,y,z)
// plus a count of non-finite coordinates.
__global__ void k_bbox(const float* __restrict__ xyz, uint64_t n, uint32_t* out) {
  uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0, 0, 0};
  uint32_t bad = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float v = xyz[3 * i + k];
      if (!isfinite(v)) { ++bad; continue; }
      const uint32_t o = f2o(v);
      mn[k] = min(mn[k], o);
      mx[k] = max(mx[k], o);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o; o >>= 1) {
      mn[k] = min(mn[k], __shfl_xor_sync(FULL, mn[k], o));
      mx[k] = max(mx[k], __shfl_xor_sync(FULL, mx[k], o));
    }
  }
  for (int o = 16; o; o >>= 1) bad += __shfl_xor_sync(FULL, bad, o);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) { atomicMin(&out[k], mn[k]); atomicMax(&out[3 + k], mx[k]); }
    if (bad) atomicAdd(&out[6], bad);
  }
}

__device__ __forceinline__ float be2f(uint32_t u) { return __uint_as_float(__byte_perm(u, 0, 0x0123)); }

// POS ingest: byte swap (src/PARAPROBE_EPOSEndianness.h:54-79) and ranging
// (PeriodicTable::mq2ionname, src/PARAPROBE_PeriodicTable.cpp:65-91: the first
// range with !(mq < lo) && !(mq > hi) in type order wins, else type 0).
__global__ void k_decode_pos(const uint4* __restrict__ rec, uint64_t n, const float* __restrict__ lo,
                             const float* __restrict__ hi, const uint8_t* __restrict__ ty, int nr,
                             float* __restrict__ xyz, uint8_t* __restrict__ label) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 r = rec[i];
    xyz[3 * i] = be2f(r.x);
    xyz[3 * i + 1] = be2f(r.y);
    xyz[3 * i + 2] = be2f(r.z);
    const float mq = be2f(r.w);
    uint8_t t = 0;
    for (int k = 0; k < nr; ++k) {
      if (!(mq < lo[k]) && !(mq > hi[k])) { t = ty[k]; break; }
    }
    label[i] = t;
  }
}

// -------------------------------------------------------------------- K1 grid
__device__ __forceinline__ int cell_coord(float v, float lo, float inv_h, int n) {
  int c = (int)floorf((v - lo) * inv_h);
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

__global__ void k_cell_count(const float* __restrict__ xyz, uint64_t n, Grid g, uint32_t* __restrict__ cell_of,
                             uint32_t* __restrict__ rank, uint32_t* __restrict__ counts) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const int cx = cell_coord(xyz[3 * i], g.lox, g.inv_h, g.nx);
    const int cy = cell_coord(xyz[3 * i + 1], g.loy, g.inv_h, g.ny);
    const int cz = cell_coord(xyz[3 * i + 2], g.loz, g.inv_h, g.nz);
    const uint32_t c = ((uint32_t)cz * (uint32_t)g.ny + (uint32_t)cy) * (uint32_t)g.nx + (uint32_t)cx;
    cell_of[i] = c;
    rank[i] = atomicAdd(&counts[c], 1u);
  }
}

// Three-phase exclusive scan: per-block scan (4 items per thread), scan of the
// block sums (recursively), add-back.
constexpr int SCAN_T = 512, SCAN_I = 4, SCAN_B = SCAN_T * SCAN_I;

template <typename T>
__device__ T block_excl_scan(T v, T* warp_sums, T* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(FULL, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sums[w] = inc;
  __syncthreads();
  if (w == 0) {
    T s = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : T(0);
    T si = s;
    for (int o = 1; o < 32; o <<= 1) {
      const T t = __shfl_up_sync(FULL, si, o);
      if (lane >= o) si += t;
    }
    warp_sums[lane] = si - s;
    if (lane == 31) *total = si;
  }
  __syncthreads();
  return warp_sums[w] + inc - v;
}

template <typename T>
__global__ void k_prefix_blocks(T* data, uint64_t n, T* block_sums) {
  __shared__ T ws[32];
  __shared__ T tot;
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_B + (uint64_t)threadIdx.x * SCAN_I;
  T v[SCAN_I];
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_I; ++k) { v[k] = (base + k < n) ? data[base + k] : T(0); s += v[k]; }
  T off = block_excl_scan<T>(s, ws, &tot);
#pragma unroll
  for (int k = 0; k < SCAN_I; ++k) {
    if (base + k < n) data[base + k] = off;
    off += v[k];
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void k_prefix_add(T* data, uint64_t n, const T* block_off) {
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_B + (uint64_t)threadIdx.x * SCAN_I;
  const T o = block_off[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_I; ++k)
    if (base + k < n) data[base + k] += o;
}

void scan_launched(int k);

template <typename T>
static void excl_scan(T* data, uint64_t n, T* tmp, uint64_t tmp_elems, cudaStream_t s) {
  const uint64_t nb = (n + SCAN_B - 1) / SCAN_B;
  if (nb == 0) return;
  k_prefix_blocks<T><<<(unsigned)nb, SCAN_T, 0, s>>>(data, n, tmp);
  scan_launched(1);
  if (nb > 1) {
    excl_scan<T>(tmp, nb, tmp + nb, tmp_elems - nb, s);
    k_prefix_add<T><<<(unsigned)nb, SCAN_T, 0, s>>>(data, n, tmp);
    scan_launched(1);
  }
}

__global__ void k_u32_to_u64(const uint32_t* in, uint64_t n, unsigned long long* out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

__global__ void k_scatter(const float* __restrict__ xyz, const uint8_t* __restrict__ label, uint64_t n,
                          const uint32_t* __restrict__ cell_of, const uint32_t* __restrict__ rank,
                          const uint32_t* __restrict__ cell_start, float4* __restrict__ ions,
                          uint32_t* __restrict__ slot_of_id, uint32_t* __restrict__ id_of_slot) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t slot = cell_start[cell_of[i]] + rank[i];
    const uint32_t lab = label[i];
    ions[slot] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], __uint_as_float(lab));
    slot_of_id[i] = slot;
    id_of_slot[slot] = (uint32_t)i;
  }
}

// The labels in slot order from the records' fourth word: a coalesced pass
// after the scatter, which thereby avoids a scattered one-byte store per ion.
__global__ void k_labels_of_ions(const float4* __restrict__ ions, uint64_t n, uint8_t* __restrict__ label_sorted) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    label_sorted[i] = (uint8_t)__float_as_uint(ions[i].w);
}

// label sets given in input order -> sorted-slot order, nsets arrays at once
__global__ void k_gather_labels(const uint8_t* __restrict__ src, const uint32_t* __restrict__ id_of_slot,
                                uint64_t n, uint8_t* __restrict__ dst, int nsets) {
  const uint64_t total = n * (uint64_t)nsets;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = t / n, slot = t - r * n;
    dst[t] = src[r * n + id_of_slot[slot]];
  }
}

// shuffled label of ion i = label[perm[i]]; written in sorted-slot order
__global__ void k_permute_labels(const uint8_t* __restrict__ label_by_id, const uint32_t* __restrict__ perm,
                                 const uint32_t* __restrict__ id_of_slot, uint64_t n, uint8_t* __restrict__ dst) {
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t id = id_of_slot[s];
    const uint32_t src = perm[id];
    dst[s] = (src < n) ? label_by_id[src] : 0;
  }
}

// ------------------------------------------------------------------- K2 hull
__device__ __forceinline__ float clamp01(float x) {
  const float lo = (x < 0.f) ? 0.f : x;  // MAX(x, 0.f) of src/PARAPROBE_Abinitio.h:48
  return (lo < 1.f) ? lo : 1.f;           // MIN(., 1.f)
}

// Squared distance to the closest point of a triangle: the region analysis of
// D. Eberly, "Distance Between Point and Triangle in 3D", evaluated in the
// order of src/PARAPROBE_Math.cpp:88-184 (region-6 fallback included).
__device__ float tri_dist2(const float* __restrict__ t, float px, float py, float pz) {
  const float e0x = __fsub_rn(t[3], t[0]), e0y = __fsub_rn(t[4], t[1]), e0z = __fsub_rn(t[5], t[2]);
  const float e1x = __fsub_rn(t[6], t[0]), e1y = __fsub_rn(t[7], t[1]), e1z = __fsub_rn(t[8], t[2]);
  const float vx = __fsub_rn(t[0], px), vy = __fsub_rn(t[1], py), vz = __fsub_rn(t[2], pz);
  const float a = __fadd_rn(__fadd_rn(__fmul_rn(e0x, e0x), __fmul_rn(e0y, e0y)), __fmul_rn(e0z, e0z));
  const float b = __fadd_rn(__fadd_rn(__fmul_rn(e0x, e1x), __fmul_rn(e0y, e1y)), __fmul_rn(e0z, e1z));
  const float c = __fadd_rn(__fadd_rn(__fmul_rn(e1x, e1x), __fmul_rn(e1y, e1y)), __fmul_rn(e1z, e1z));
  const float d = __fadd_rn(__fadd_rn(__fmul_rn(e0x, vx), __fmul_rn(e0y, vy)), __fmul_rn(e0z, vz));
  const float e = __fadd_rn(__fadd_rn(__fmul_rn(e1x, vx), __fmul_rn(e1y, vy)), __fmul_rn(e1z, vz));
  const float det = __fsub_rn(__fmul_rn(a, c), __fmul_rn(b, b));
  float s = __fsub_rn(__fmul_rn(b, e), __fmul_rn(c, d));
  float u = __fsub_rn(__fmul_rn(b, d), __fmul_rn(a, e));
  if (__fadd_rn(s, u) < det) {
    if (s < 0.f) {
      if (u < 0.f) {
        if (d < 0.f) { s = clamp01(__fdiv_rn(-d, a)); u = 0.f; }
        else { s = 0.f; u = clamp01(__fdiv_rn(-e, c)); }
      } else { s = 0.f; u = clamp01(__fdiv_rn(-e, c)); }
    } else if (u < 0.f) {
      s = clamp01(__fdiv_rn(-d, a)); u = 0.f;
    } else {
      const float inv = __fdiv_rn(1.f, det);
      s = __fmul_rn(s, inv); u = __fmul_rn(u, inv);
    }
  } else {
    const float den = __fadd_rn(__fsub_rn(a, __fmul_rn(2.f, b)), c);
    if (s < 0.f) {
      const float t0 = __fadd_rn(b, d), t1 = __fadd_rn(c, e);
      if (t1 > t0) { s = clamp01(__fdiv_rn(__fsub_rn(t1, t0), den)); u = __fsub_rn(1.f, s); }
      else { u = clamp01(__fdiv_rn(-e, c)); s = 0.f; }
    } else if (u < 0.f) {
      if (__fadd_rn(a, d) > __fadd_rn(b, e)) {
        const float num = __fsub_rn(__fsub_rn(__fadd_rn(c, e), b), d);
        s = clamp01(__fdiv_rn(num, den)); u = __fsub_rn(1.f, s);
      } else { s = clamp01(__fdiv_rn(-e, c)); u = 0.f; }
    } else {
      const float num = __fsub_rn(__fsub_rn(__fadd_rn(c, e), b), d);
      s = clamp01(__fdiv_rn(num, den)); u = __fsub_rn(1.f, s);
    }
  }
  const float cx = __fadd_rn(__fadd_rn(t[0], __fmul_rn(s, e0x)), __fmul_rn(u, e1x));
  const float cy = __fadd_rn(__fadd_rn(t[1], __fmul_rn(s, e0y)), __fmul_rn(u, e1y));
  const float cz = __fadd_rn(__fadd_rn(t[2], __fmul_rn(s, e0z)), __fmul_rn(u, e1z));
  const float qx = __fsub_rn(cx, px), qy = __fsub_rn(cy, py), qz = __fsub_rn(cz, pz);
  return __fadd_rn(__fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy)), __fmul_rn(qz, qz));
}

// ion2surf per sorted slot: R'^2, lowered to the smallest tri_dist2 over the
// triangles whose float AABB overlaps [p - R', p + R'] (touching counts,
// src/PARAPROBE_AABBTree.cpp:112-124), in the order of the cell's list; every
// triangle is listed in each hull cell its AABB grown by R' + slack reaches.
// One warp per hull cell: the hull grid `tg` is the
// ion grid `g` coarsened f times per axis (same origin), so a hull cell's ions
// are f x f row segments of consecutive slots.  The warp takes them 32 at a
// time (rows concatenated); the cell's triangles are staged in shared memory
// 32 at a time (box and vertices, loaded by the lanes together) and every
// lane tests them against its own ion in list order (an ion per thread
// walking its own list took 25% longer: lanes of a warp span several hull
// cells, and each triangle was a chain of dependent global loads).  The ion's
// hull cell (its ion cell divided by f) lists every triangle whose box grown
// by R' + slack reaches it: the two cell computations can only disagree
// within float rounding of a boundary, which the slack covers.
constexpr int kSurfWarps = 8;
__global__ void __launch_bounds__(kSurfWarps * 32) k_surface_cells(const float4* __restrict__ ions,
                                                              const uint32_t* __restrict__ cell_start, Grid g, int f,
                                                              const float* __restrict__ tbox,
                                                              const float* __restrict__ tri,
                                                              const uint32_t* __restrict__ tstart,
                                                              const uint32_t* __restrict__ tlist, Grid tg, float rp,
                                                              float* __restrict__ out) {
  // per staged triangle: box lo x,y,z, hi x,y,z, the 9 vertex coordinates and
  // a pad (17 words: conflict-free stores)
  __shared__ float stri[kSurfWarps][32][17];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float (*st)[17] = stri[warp];
  const uint32_t lemask = (2u << lane) - 1u;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const float rp2 = __fmul_rn(rp, rp);
  for (uint64_t tc = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; tc < tg.ncells; tc += nwarps) {
    const int tx = (int)(tc % (uint64_t)tg.nx);
    const uint64_t tr = tc / (uint64_t)tg.nx;
    const int ty = (int)(tr % (uint64_t)tg.ny), tz = (int)(tr / (uint64_t)tg.ny);
    const uint32_t k0 = tstart[tc], k1 = tstart[tc + 1];
    const int x0 = tx * f, x1 = min(x0 + f, g.nx);
    const int ny = min(f, g.ny - ty * f), nz = min(f, g.nz - tz * f);
    const int nrows = ny * nz;
    for (int r0 = 0; r0 < nrows; r0 += 32) {
      // row r0 + lane: its slots; then the rows with ions, concatenated
      uint32_t st0 = 0, len = 0;
      if (r0 + lane < nrows) {
        const int yy = ty * f + (r0 + lane) % ny, zz = tz * f + (r0 + lane) / ny;
        const uint64_t rowb = ((uint64_t)zz * g.ny + yy) * g.nx;
        st0 = cell_start[rowb + x0];
        len = cell_start[rowb + x1] - st0;
      }
      const uint32_t ne = __ballot_sync(FULL, len > 0);
      const int cnt_rows = __popc(ne);
      if (cnt_rows == 0) continue;
      const int src = lane < cnt_rows ? (int)__fns(ne, 0, lane + 1) : 0;
      const uint32_t rst = __shfl_sync(FULL, st0, src);
      uint32_t rlen = __shfl_sync(FULL, len, src);
      if (lane >= cnt_rows) rlen = 0;
      uint32_t inc = rlen;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += t;
      }
      const uint32_t exc = inc - rlen;
      const uint32_t total = __shfl_sync(FULL, inc, 31);
      int before = 0;
      for (uint32_t bb = 0; bb < total; bb += 32) {
        const uint32_t bitv = (lane < cnt_rows && rlen > 0 && exc >= bb && exc < bb + 32) ? (1u << (exc - bb)) : 0u;
        const uint32_t smask = __reduce_or_sync(FULL, bitv);
        const int row = before + __popc(smask & lemask) - 1;
        before += __popc(smask);
        const int rowc = row < 0 ? 0 : (row > 31 ? 31 : row);
        const uint32_t rs = __shfl_sync(FULL, rst, rowc);
        const uint32_t rpos = __shfl_sync(FULL, exc, rowc);
        const uint32_t t = bb + lane;
        const bool have = t < total;
        const uint32_t slot = rs + (t - rpos);
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        if (have) p = ions[slot];
        float best = rp2;
        const float lx = __fsub_rn(p.x, rp), ly = __fsub_rn(p.y, rp), lz = __fsub_rn(p.z, rp);
        const float hx = __fadd_rn(p.x, rp), hy = __fadd_rn(p.y, rp), hz = __fadd_rn(p.z, rp);
        for (uint32_t kb = k0; kb < k1; kb += 32) {
          if (kb + lane < k1) {
            const uint32_t tt = tlist[kb + lane];
            const float* b = tbox + 6 * (uint64_t)tt;
            const float* v = tri + 9 * (uint64_t)tt;
#pragma unroll
            for (int q = 0; q < 6; ++q) st[lane][q] = b[q];
#pragma unroll
            for (int q = 0; q < 9; ++q) st[lane][6 + q] = v[q];
          }
          __syncwarp();
          const int m = (int)min(32u, k1 - kb);
          for (int j = 0; j < m; ++j) {
            const float* b = st[j];
            if (!have || b[3] < lx || b[0] > hx || b[4] < ly || b[1] > hy || b[5] < lz || b[2] > hz) continue;
            const float v = tri_dist2(b + 6, p.x, p.y, p.z);
            if (!(v > best)) best = v;
          }
          __syncwarp();
        }
        if (have) out[slot] = best;
      }
    }
  }
}

// Occupancy grid behind the RDF header: voxel of every ion as
// threadmemory::rectangular_transfer computes it (src/PARAPROBE_SolverHdl.cpp:
// 1471-1508): t = (p - lo) / w in float, voxel 1 + (size_t)t unless that
// truncation lands on the last voxel.  Counts ions per voxel.
__global__ void k_voxel_count(const float* __restrict__ xyz, uint64_t n, float lox, float loy, float loz, float w,
                              uint32_t nx, uint32_t ny, uint32_t nz, uint32_t* __restrict__ occ, int* status) {
  const float lo[3] = {lox, loy, loz};
  const uint64_t nv[3] = {nx, ny, nz};
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float t = __fdiv_rn(__fsub_rn(xyz[3 * i + k], lo[k]), w);
      const uint64_t sz = (uint64_t)t;
      c[k] = (sz != nv[k] - 1) ? 1 + sz : nv[k] - 1;
    }
    if (c[0] >= nx || c[1] >= ny || c[2] >= nz) {  // cannot happen for a box that holds the cloud
      atomicOr(status, ST_BAD_SLOT);
      continue;
    }
    atomicAdd(&occ[c[0] + c[1] * nx + c[2] * (uint64_t)nx * ny], 1u);
  }
}

// Caller-order variant for the entry point without allocations: positions as
// packed xyz triples and ion2surf written in the same order.  The candidate
// test and the minimum are those of k_surface_cells, so both give the same bits.
__global__ void k_surface_xyz(const float* __restrict__ xyz, uint64_t n, const float* __restrict__ tbox,
                              const float* __restrict__ tri, const uint32_t* __restrict__ tstart,
                              const uint32_t* __restrict__ tlist, Grid tg, float rp, float* __restrict__ out) {
  const float rp2 = __fmul_rn(rp, rp);
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
    float best = rp2;
    const int cx = (int)floorf((px - tg.lox) * tg.inv_h), cy = (int)floorf((py - tg.loy) * tg.inv_h),
              cz = (int)floorf((pz - tg.loz) * tg.inv_h);
    if (cx >= 0 && cy >= 0 && cz >= 0 && cx < tg.nx && cy < tg.ny && cz < tg.nz) {
      const uint64_t c = ((uint64_t)cz * tg.ny + cy) * tg.nx + cx;
      const float lx = __fsub_rn(px, rp), ly = __fsub_rn(py, rp), lz = __fsub_rn(pz, rp);
      const float hx = __fadd_rn(px, rp), hy = __fadd_rn(py, rp), hz = __fadd_rn(pz, rp);
      const uint32_t k1 = tstart[c + 1];
      for (uint32_t k = tstart[c]; k < k1; ++k) {
        const uint32_t t = tlist[k];
        const float* b = tbox + 6 * (uint64_t)t;
        if (b[3] < lx || b[0] > hx || b[4] < ly || b[1] > hy || b[5] < lz || b[2] > hz) continue;
        const float v = tri_dist2(tri + 9 * (uint64_t)t, px, py, pz);
        if (!(v > best)) best = v;
      }
    }
    out[i] = best;
  }
}

// Triangle boxes on the device: per axis the smallest and largest vertex
// coordinate (lo x,y,z then hi x,y,z), for the hull cell lists and distances.
__global__ void k_tri_box(const float* __restrict__ tri, uint64_t ntri, float* __restrict__ box) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ntri; t += (uint64_t)gridDim.x * blockDim.x) {
    const float* v = tri + 9 * t;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      box[6 * t + k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
      box[6 * t + 3 + k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
    }
  }
}

// --------------------------------------------------------- centre selection
// Centre filter of src/PARAPROBE_SolverHdl.cpp:3847-3859: the type is a target
// of some task and ion2surf >= R^2 (plus an optional extra mask).  The
// compaction keeps cell order (flags, exclusive scan, write), so consecutive
// centres are spatial neighbours and a block's warps share stencil rows in L1.
__device__ __forceinline__ bool centre_ok(const uint8_t* labels, const float* surf, uint64_t i, float R2,
                                          const int8_t* cslot_of, const uint8_t* extra) {
  const bool target = cslot_of ? (cslot_of[labels[i]] >= 0) : true;
  return target && (surf[i] >= R2) && (extra ? extra[i] != 0 : true);
}

__global__ void k_select_flags(const uint8_t* __restrict__ labels, const float* __restrict__ surf, uint64_t n,
                               float R2, const int8_t* __restrict__ cslot_of, const uint8_t* __restrict__ extra,
                               uint32_t* __restrict__ flags, uint8_t* __restrict__ cflag) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= n; i += (uint64_t)gridDim.x * blockDim.x) {
    const bool ok = i < n && centre_ok(labels, surf, i, R2, cslot_of, extra);
    flags[i] = ok ? 1u : 0u;
    if (cflag && i < n) cflag[i] = ok ? 1 : 0;
  }
}

// Number of non-centre ions per cell (for the symmetric pass's row skipping).
__global__ void k_nc_count(const uint32_t* __restrict__ cell_start, uint64_t ncells, const uint8_t* __restrict__ cflag,
                           uint32_t* __restrict__ out) {
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c <= ncells; c += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t k = 0;
    if (c < ncells)
      for (uint32_t j = cell_start[c]; j < cell_start[c + 1]; ++j) k += cflag[j] ? 0u : 1u;
    out[c] = k;
  }
}

// Triangle binning for the hull distance: every cell of tg that a triangle's
// box grown by `grow` touches lists the triangle (count, scan, fill).
__device__ __forceinline__ void tri_cell_range(const float* b, Grid tg, float grow, int* c0, int* c1) {
  const float org[3] = {tg.lox, tg.loy, tg.loz};
  const int nmax[3] = {tg.nx, tg.ny, tg.nz};
  for (int k = 0; k < 3; ++k) {
    int lo = (int)floorf((b[k] - grow - org[k]) * tg.inv_h);
    int hi = (int)floorf((b[3 + k] + grow - org[k]) * tg.inv_h);
    c0[k] = lo < 0 ? 0 : (lo >= nmax[k] ? nmax[k] - 1 : lo);
    c1[k] = hi < 0 ? 0 : (hi >= nmax[k] ? nmax[k] - 1 : hi);
    // a grown box wholly beyond the grid (which covers every ion) reaches no ion
    if (hi < 0 || lo >= nmax[k]) { c0[k] = 1; c1[k] = 0; }
  }
}

// A warp per triangle, its lanes over the cells of the triangle's range (a
// triangle reaches tens of cells; one thread walking them all left the list
// fill latency-bound on its chain of returning atomics).
__device__ __forceinline__ uint64_t tri_range_cell(const Grid& tg, const int* c0, const int* c1, uint32_t i) {
  const uint32_t nx = (uint32_t)(c1[0] - c0[0] + 1), ny = (uint32_t)(c1[1] - c0[1] + 1);
  const int x = c0[0] + (int)(i % nx), y = c0[1] + (int)((i / nx) % ny), z = c0[2] + (int)(i / (nx * ny));
  return ((uint64_t)z * tg.ny + y) * tg.nx + x;
}

__global__ void k_tri_count(const float* __restrict__ tbox, uint64_t ntri, Grid tg, float grow,
                            uint32_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; t < ntri; t += nw) {
    int c0[3], c1[3];
    tri_cell_range(tbox + 6 * t, tg, grow, c0, c1);
    const uint32_t m = (uint32_t)(c1[0] - c0[0] + 1) * (uint32_t)(c1[1] - c0[1] + 1) * (uint32_t)(c1[2] - c0[2] + 1);
    for (uint32_t i = lane; i < m; i += 32) atomicAdd(&cnt[tri_range_cell(tg, c0, c1, i)], 1u);
  }
}

__global__ void k_tri_fill(const float* __restrict__ tbox, uint64_t ntri, Grid tg, float grow,
                           uint32_t* __restrict__ fill, uint32_t* __restrict__ list, uint64_t cap,
                           int* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; t < ntri; t += nw) {
    int c0[3], c1[3];
    tri_cell_range(tbox + 6 * t, tg, grow, c0, c1);
    const uint32_t m = (uint32_t)(c1[0] - c0[0] + 1) * (uint32_t)(c1[1] - c0[1] + 1) * (uint32_t)(c1[2] - c0[2] + 1);
    for (uint32_t i = lane; i < m; i += 32) {
      const uint32_t at = atomicAdd(&fill[tri_range_cell(tg, c0, c1, i)], 1u);
      if (at < cap) list[at] = (uint32_t)t;
      else if (status) atomicOr(status, ST_LIST_OVERFLOW);
    }
  }
}

// Number of (triangle, cell) list entries binning into tg would make, in 64
// bits, so that a grid is only filled when its lists fit the space at hand.
__global__ void k_tri_entries(const float* __restrict__ tbox, uint64_t ntri, Grid tg, float grow,
                              unsigned long long* total) {
  unsigned long long sum = 0;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ntri; t += (uint64_t)gridDim.x * blockDim.x) {
    int c0[3], c1[3];
    tri_cell_range(tbox + 6 * t, tg, grow, c0, c1);
    sum += (unsigned long long)(c1[0] - c0[0] + 1) * (c1[1] - c0[1] + 1) * (c1[2] - c0[2] + 1);
  }
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(total, sum);
}


__global__ void k_select_write(const uint8_t* __restrict__ labels, const float* __restrict__ surf, uint64_t n,
                               float R2, const int8_t* __restrict__ cslot_of, const uint8_t* __restrict__ extra,
                               const uint32_t* __restrict__ pos, uint32_t* __restrict__ out,
                               uint32_t* __restrict__ count) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (centre_ok(labels, surf, i, R2, cslot_of, extra)) out[pos[i]] = (uint32_t)i;
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = pos[n];
}

// --------------------------------------------------------------- K3 the scan
// Row offsets (dy, dz) of stencils with half-width s = 0..ROW_SMAX, each table
// sorted by dy^2 + dz^2; table s starts at entry row_table_offset(s) =
// sum_{t<s} (2t+1)^2 (built on the host, copied to shared memory).
constexpr int ROW_SMAX = 7;
__host__ __device__ constexpr int row_table_offset(int s) { return s * (4 * s * s - 1) / 3; }
constexpr int ROW_TABLE_ENTRIES = row_table_offset(ROW_SMAX + 1);

__device__ __forceinline__ int category(float d2, const float* __restrict__ sT, int H, float gs, float gk) {
  int g = (int)((sqrtf(d2) - gs) * gk) + 1;
  g = g < 0 ? 0 : (g > H - 1 ? H - 1 : g);
  while (g + 1 < H && sT[g + 1] <= d2) ++g;
  while (g > 0 && sT[g] > d2) --g;
  return g;
}

// The same category from the lookup table: start at the category of the
// table cell's smallest d^2 and step up through the thresholds.
__device__ __forceinline__ int category_lut(float d2, const uint16_t* __restrict__ lut, int lut_n, uint32_t lut_base,
                                            int lut_shift, const float* __restrict__ sT, int H) {
  int idx = (int)(__float_as_uint(d2) >> lut_shift) - (int)lut_base;
  idx = idx < 0 ? 0 : (idx >= lut_n ? lut_n - 1 : idx);
  int g = lut[idx];
  while (g + 1 < H && sT[g + 1] <= d2) ++g;
  return g;
}

// The same category for an in-ball d^2 (d^2 <= R^2) when every table cell
// below R^2 holds at most one threshold (ScanArgs::lut_one, checked by the
// host): the cell's category plus one branch-free step.  T holds +inf at H.
__device__ __forceinline__ int category_one(float d2, const uint16_t* __restrict__ lut, int lut_n, uint32_t lut_base,
                                            int lut_shift, const float* __restrict__ T) {
  int t = (int)(__float_as_uint(d2) >> lut_shift) - (int)lut_base;
  t = t < 0 ? 0 : (t >= lut_n ? lut_n - 1 : t);
  const int g = lut[t];
  return g + (T[g + 1] <= d2 ? 1 : 0);
}

template <int KR>
__device__ __forceinline__ void list_insert(float (&l)[KR], float x, int lane) {
  int pos = 0;
#pragma unroll
  for (int r = 0; r < KR; ++r) pos += __popc(__ballot_sync(FULL, l[r] <= x));
  float prev[KR];
#pragma unroll
  for (int r = 0; r < KR; ++r) {
    const float up = __shfl_up_sync(FULL, l[r], 1);
    const float carry = (r > 0) ? __shfl_sync(FULL, l[r > 0 ? r - 1 : 0], 31) : 0.f;
    prev[r] = (lane == 0) ? carry : up;
  }
#pragma unroll
  for (int r = 0; r < KR; ++r) {
    const int idx = r * 32 + lane;
    if (idx > pos) l[r] = prev[r];
    else if (idx == pos) l[r] = x;
  }
}

// element e = row * 32 + src of the distributed list (row, src may differ per lane)
template <int KR>
__device__ __forceinline__ float list_get(const float (&l)[KR], int row, int src) {
  float v = 0.f;
#pragma unroll
  for (int r = 0; r < KR; ++r) {
    const float t = __shfl_sync(FULL, l[r], src);
    if (r == row) v = t;
  }
  return v;
}

struct ScanShared {
  int8_t* rowtab; // [ROW_TABLE_ENTRIES][2]
  uint16_t* lut;  // [lut_n] category lookup
  float* lst;     // [warps][emax][LS] sorted kNN lists (disjoint sets)
  float* T;
  int8_t* cs;
  int8_t* es;
  int8_t* sidx;   // [nC][256] the only env set of a type, or -1 (disjoint sets)
  uint32_t* env;
  uint32_t* rdf;
  uint32_t* cnt;
  int* hist;  // mode 2: per-warp category histogram
  unsigned long long* since_flush;
};

// Iterates the candidates of one centre: every ion of every stencil row
// (y, z) whose cells can hold a point within R + margin, with the row's x
// range trimmed to the ball.  Rows are compacted and their ions streamed 32 at
// a time across the warp; f(valid, slot, d2, inball, type) is called
// warp-uniformly once per 32 candidates.
template <class F>
__device__ __forceinline__ void for_each_candidate_r(const ScanArgs& a, const int8_t* __restrict__ rowtab, float4 cp,
                                                     uint32_t self, int lane, float R, float Rm2, float R2, F&& f) {
  const Grid& g = a.g;
  const float ext = R + g.margin;
  auto clampc = [](int c, int n) { return c < 0 ? 0 : (c >= n ? n - 1 : c); };
  const int y0 = clampc((int)floorf((cp.y - ext - g.loy) * g.inv_h), g.ny);
  const int y1 = clampc((int)floorf((cp.y + ext - g.loy) * g.inv_h), g.ny);
  const int z0 = clampc((int)floorf((cp.z - ext - g.loz) * g.inv_h), g.nz);
  const int z1 = clampc((int)floorf((cp.z + ext - g.loz) * g.inv_h), g.nz);
  const int yc = clampc((int)floorf((cp.y - g.loy) * g.inv_h), g.ny);
  const int zc = clampc((int)floorf((cp.z - g.loz) * g.inv_h), g.nz);
  const int xc = clampc((int)floorf((cp.x - g.lox) * g.inv_h), g.nx);
  // rows are visited in order of increasing offset from the centre's row, so
  // the nearest candidates come first (the kNN lists settle early)
  int sr = max(max(yc - y0, y1 - yc), max(zc - z0, z1 - zc));
  if (sr > ROW_SMAX) {  // cannot happen for cell edges >= R / 6; recorded, never silent
    if (lane == 0) atomicOr(a.status, ST_BAD_SLOT);
    sr = ROW_SMAX;
  }
  const int nrows = (2 * sr + 1) * (2 * sr + 1);
  const int8_t* tab = rowtab + 2 * row_table_offset(sr);
  const uint32_t lemask = (2u << lane) - 1u;
  for (int r0 = 0; r0 < nrows; r0 += 32) {
    const int r = r0 + lane;
    uint32_t st = 0, len = 0;
    const int yy = (r < nrows) ? yc + tab[2 * r] : -1;
    const int zz = (r < nrows) ? zc + tab[2 * r + 1] : -1;
    if (r < nrows && yy >= y0 && yy <= y1 && zz >= z0 && zz <= z1) {
      const float ylo = g.loy + (float)yy * g.h - g.margin, yhi = g.loy + (float)(yy + 1) * g.h + g.margin;
      const float zlo = g.loz + (float)zz * g.h - g.margin, zhi = g.loz + (float)(zz + 1) * g.h + g.margin;
      const float dy = fmaxf(0.f, fmaxf(ylo - cp.y, cp.y - yhi));
      const float dz = fmaxf(0.f, fmaxf(zlo - cp.z, cp.z - zhi));
      const float rem = Rm2 - dy * dy - dz * dz;
      if (rem >= 0.f) {
        const float half = sqrtf(rem) + g.margin;
        const int x0 = clampc((int)floorf((cp.x - half - g.lox) * g.inv_h), g.nx);
        const int x1 = clampc((int)floorf((cp.x + half - g.lox) * g.inv_h), g.nx);
        const uint64_t cb = ((uint64_t)zz * g.ny + yy) * g.nx;
        int xs = x0;
        if (a.sym) {
          // cells that precede the centre in slot order and hold only centres
          // are skipped: each of those pairs is taken by the other centre
          const bool own = (zz == zc && yy == yc);
          if (own || zz < zc || (zz == zc && yy < yc)) {
            const int xe = own ? min(x1, xc - 1) : x1;
            if (xe >= x0 && a.nc_pre[cb + xe + 1] == a.nc_pre[cb + x0]) xs = xe + 1;
          }
        }
        if (xs <= x1) {
          st = a.cell_start[cb + xs];
          len = a.cell_start[cb + x1 + 1] - st;
        }
      }
    }
    const uint32_t ne = __ballot_sync(FULL, len > 0);
    const int cnt = __popc(ne);
    if (cnt == 0) continue;
    const int src = (lane < cnt) ? (int)__fns(ne, 0, lane + 1) : 0;
    const uint32_t rst = __shfl_sync(FULL, st, src);
    uint32_t rlen = __shfl_sync(FULL, len, src);
    if (lane >= cnt) rlen = 0;
    uint32_t inc = rlen;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(FULL, inc, o);
      if (lane >= o) inc += t;
    }
    const uint32_t exc = inc - rlen;
    const uint32_t total = __shfl_sync(FULL, inc, 31);
    int before = 0;
    for (uint32_t b = 0; b < total; b += 32) {
      const uint32_t bitv = (lane < cnt && rlen > 0 && exc >= b && exc < b + 32) ? (1u << (exc - b)) : 0u;
      const uint32_t sm = __reduce_or_sync(FULL, bitv);
      const int row = before + __popc(sm & lemask) - 1;
      before += __popc(sm);
      const int rowc = row < 0 ? 0 : (row > 31 ? 31 : row);
      const uint32_t rs = __shfl_sync(FULL, rst, rowc);
      const uint32_t rp = __shfl_sync(FULL, exc, rowc);
      const uint32_t t = b + lane;
      const bool valid = t < total;
      const uint32_t slot = rs + (t - rp);
      float d2 = kInf();
      uint32_t m = 0;
      bool inball = false, jcentre = false;
      if (valid) {
        const float4 q = __ldg(a.ions + slot);
        d2 = dist2(cp.x, cp.y, cp.z, q.x, q.y, q.z);
        // symmetric mode: a pair of two centres is taken once, by the lower slot
        if (a.sym) jcentre = a.cflag[slot] != 0;
        inball = (d2 <= R2) && (slot != self) && !(jcentre && slot < self);
        m = a.labels ? (uint32_t)a.labels[slot] : __float_as_uint(q.w);
      }
      f(valid, slot, d2, inball, m, jcentre && slot > self);
    }
  }
}

// The same walk at the pass's radius (ScanArgs::R, Rm2, R2).
template <class F>
__device__ __forceinline__ void for_each_candidate(const ScanArgs& a, const int8_t* __restrict__ rowtab, float4 cp,
                                                   uint32_t self, int lane, F&& f) {
  for_each_candidate_r(a, rowtab, cp, self, lane, a.R, a.Rm2, a.R2, f);
}

template <int KR, int EMAX>
__global__ void __launch_bounds__(256) k_scan(ScanArgs a) {
  // shared kNN list stride: one padding word keeps set p's k-th entry in bank
  // (p + k) % 32, so lanes testing different sets do not collide
  constexpr int LS = (KR > 0 ? KR : 1) * 32 + 1;
  extern __shared__ __align__(16) unsigned char smem[];
  const int H = a.H;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  ScanShared S;
  {
    unsigned char* p = smem;
    S.since_flush = (unsigned long long*)p; p += 16;
    S.rowtab = (int8_t*)p; p += ROW_TABLE_ENTRIES * 2;
    S.T = (float*)p; p += ((H + 4) & ~3) * 4;  // H thresholds, then +inf
    S.lut = (uint16_t*)p; p += ((a.lut_n + 7) & ~7) * 2;
    S.cs = (int8_t*)p; p += 256;
    S.es = (int8_t*)p; p += 256;
    S.env = (uint32_t*)p; p += (KR > 0 ? a.nC * 256 * 4 : 0);
    S.lst = (float*)p; p += ((KR > 0 && a.disjoint) ? nwarps * a.emax * LS * 4 : 0);
    S.rdf = (uint32_t*)p; p += (a.rdf_in_smem ? a.nC * a.nE * H * 4 : 0);
    S.cnt = (uint32_t*)p; p += ((a.flags & PP_CNTNB) ? nwarps * a.nE * 4 : 0);
    S.hist = (int*)p; p += (a.mode == 2 ? nwarps * H * 4 : 0);
    S.sidx = (int8_t*)p;
  }
  for (int i = threadIdx.x; i <= H; i += blockDim.x) S.T[i] = i < H ? a.cat_T[i] : kInf();
  for (int i = threadIdx.x; i < a.lut_n; i += blockDim.x) S.lut[i] = a.cat_lut[i];
  for (int i = threadIdx.x; i < ROW_TABLE_ENTRIES * 2; i += blockDim.x) S.rowtab[i] = a.rowtab[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) { S.cs[i] = a.cslot_of[i]; S.es[i] = a.eslot_of[i]; }
  if (KR > 0) for (int i = threadIdx.x; i < a.nC * 256; i += blockDim.x) S.env[i] = a.envbits[i];
  if (KR > 0 && a.disjoint) for (int i = threadIdx.x; i < a.nC * 256; i += blockDim.x) S.sidx[i] = a.setidx[i];
  if (a.rdf_in_smem) for (int i = threadIdx.x; i < a.nC * a.nE * H; i += blockDim.x) S.rdf[i] = 0;
  if (a.flags & PP_CNTNB) for (int i = threadIdx.x; i < nwarps * a.nE; i += blockDim.x) S.cnt[i] = 0;
  if (a.mode == 2) for (int i = threadIdx.x; i < nwarps * H; i += blockDim.x) S.hist[i] = 0;
  if (threadIdx.x == 0) *S.since_flush = 0ull;
  __syncthreads();

  const bool doR = (a.flags & PP_RDF) && a.mode == 0;
  const bool doC = (a.flags & PP_CNTNB) && a.mode == 0;
  const bool doK = KR > 0 && a.mode == 0;
  const int krow = (a.kmax - 1) >> 5, klane = (a.kmax - 1) & 31;
  unsigned long long pairs_lane = 0, centres = 0, tests_lane = 0;
  constexpr unsigned long long FLUSH = 1ull << 30;
  __shared__ uint32_t s_tile, s_next;
  const uint32_t T = a.tile;
  const uint32_t ntiles = (a.ncentres + T - 1) / T;

  // Work: a block takes a tile of consecutive (cell-ordered) centres from a
  // global counter; its warps take centres of the tile one at a time.
  for (;;) {
    if (threadIdx.x == 0) { s_tile = atomicAdd(a.work, 1u); s_next = 0; }
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint32_t c0 = tile * T, clen = min(T, a.ncentres - c0);
    for (;;) {
    uint32_t kk = 0;
    if (lane == 0) kk = atomicAdd(&s_next, 1u);
    kk = __shfl_sync(FULL, kk, 0);
    if (kk >= clen) break;
    {
      const uint32_t ci = c0 + kk;
      const uint32_t self = a.centres[a.sample_stride > 1 ? (uint64_t)ci * a.sample_stride : ci];
      const float4 cp = a.ions[self];
      const uint32_t ct = a.labels ? (uint32_t)a.labels[self] : __float_as_uint(cp.w);
      const int cs = (a.mode == 0) ? S.cs[ct & 255] : 0;
      if (cs < 0) {  // selection guarantees a slot; record and skip otherwise
        if (lane == 0) atomicOr(a.status, ST_TYPE_RANGE);
        continue;
      }
      uint32_t inb = 0;
      if (a.mode == 0) {
        // SL: shared-memory lists (disjoint environment sets, EMAX == 0);
        // otherwise register lists, one per local environment set
        constexpr bool SL = (EMAX == 0);
        constexpr int EM = SL ? 1 : EMAX;
        constexpr int KRR = KR > 0 ? KR : 1;
        float lst[EM][KRR];
        float thr[EM];
        int nset = 0;
        if (doK) {
          nset = a.nsets[cs];
          if constexpr (SL) {
            float* L = S.lst + warp * a.emax * LS;
            for (int e = lane; e < nset * LS; e += 32) L[e] = kInf();
            __syncwarp();
          } else {
#pragma unroll
            for (int p = 0; p < EM; ++p) {
              thr[p] = kInf();
#pragma unroll
              for (int r = 0; r < KRR; ++r) lst[p][r] = kInf();
            }
          }
        }
        for_each_candidate(a, S.rowtab, cp, self, lane,
                           [&](bool valid, uint32_t slot, float d2, bool inball, uint32_t m, bool jside) {
          (void)slot;
          tests_lane += valid ? 1u : 0u;
          if (inball) {
            ++inb;
            const int es = S.es[m & 255];
            int cat = -1;
            if (doR && es >= 0) {
              cat = a.lut_one ? category_one(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T)
                              : category_lut(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T, H);
              const uint32_t idx = ((uint32_t)cs * a.nE + es) * H + cat;
              if (a.rdf_in_smem) atomicAdd(&S.rdf[idx], 1u);
              else atomicAdd(&a.rdf_core[idx], 1ull);
            }
            if (jside) {
              // the same pair seen from neighbour j, which is a centre too
              ++inb;
              const int csj = S.cs[m & 255], esi = S.es[ct & 255];
              if (doR && esi >= 0 && csj >= 0) {
                if (cat < 0)
                  cat = a.lut_one ? category_one(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T)
                                  : category_lut(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T, H);
                const uint32_t idx = ((uint32_t)csj * a.nE + esi) * H + cat;
                if (a.rdf_in_smem) atomicAdd(&S.rdf[idx], 1u);
                else atomicAdd(&a.rdf_core[idx], 1ull);
              }
            }
            if (doC && es >= 0) atomicAdd(&S.cnt[warp * a.nE + es], 1u);
          }
          if constexpr (KR > 0 && SL) {
            if (doK) {
              // every type belongs to at most one environment set of this
              // centre type: the warp's sorted lists live in shared memory
              // (set p at L + p * LS, element e at [e]), one ballot per 32
              // candidates tests each lane against its own set's k-th value
              float* L = S.lst + warp * a.emax * LS;
              const int p = inball ? (int)S.sidx[cs * 256 + (m & 255)] : -1;
              const int kix = a.kmax - 1;
              uint32_t mask = __ballot_sync(FULL, p >= 0 && d2 < L[(p < 0 ? 0 : p) * LS + kix]);
              while (mask) {
                const int srcl = __ffs(mask) - 1;
                const float x = __shfl_sync(FULL, d2, srcl);
                const int ps = __shfl_sync(FULL, p, srcl);
                float* lp = L + ps * LS;
                float v[KR];
#pragma unroll
                for (int r = 0; r < KR; ++r) v[r] = lp[r * 32 + lane];
                list_insert<KR>(v, x, lane);
#pragma unroll
                for (int r = 0; r < KR; ++r) lp[r * 32 + lane] = v[r];
                __syncwarp();
                mask &= ~(1u << srcl);
                mask &= __ballot_sync(FULL, p >= 0 && d2 < L[(p < 0 ? 0 : p) * LS + kix]);
              }
            }
          }
          if constexpr (KR > 0 && !SL) {
            if (doK) {
              const uint32_t eb = inball ? S.env[cs * 256 + (m & 255)] : 0u;
#pragma unroll
              for (int p = 0; p < EM; ++p) {
                if (p < nset) {
                  uint32_t mask = __ballot_sync(FULL, ((eb >> p) & 1u) && d2 < thr[p]);
                  while (mask) {
                    const int srcl = __ffs(mask) - 1;
                    const float x = __shfl_sync(FULL, d2, srcl);
                    list_insert<KR>(lst[p], x, lane);
                    thr[p] = list_get<KR>(lst[p], krow, klane);
                    mask &= ~(1u << srcl);
                    mask &= __ballot_sync(FULL, d2 < thr[p]);
                  }
                }
              }
            }
          }
        });
        if constexpr (KR > 0) {
          if (doK) {
            // the k-th smallest d^2 of each set -> its bin (or the miss bin)
            auto emit = [&](int p, int kk, float v) {
              const int Sg = a.set_list[cs * 32 + p];
              const int cat = (v == kInf()) ? a.cat_miss : category_lut(v, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T, H);
              if (cat >= 0) atomicAdd(&a.knn_core[(((uint64_t)cs * a.nS + Sg) * a.nkI + kk) * H + cat], 1ull);
            };
            if constexpr (SL) {
              for (int p = 0; p < nset; ++p)
                for (int kk = lane; kk < a.nkI; kk += 32)
                  emit(p, kk, S.lst[(warp * a.emax + p) * LS + a.kvals[kk] - 1]);
            } else {
#pragma unroll
              for (int p = 0; p < EM; ++p) {
                if (p < nset) {
                  for (int k0 = 0; k0 < a.nkI; k0 += 32) {
                    const int kk = k0 + lane;
                    const int e = (kk < a.nkI) ? a.kvals[kk] - 1 : 0;
                    const float v = list_get<KR>(lst[p], e >> 5, e & 31);
                    if (kk < a.nkI) emit(p, kk, v);
                  }
                }
              }
            }
          }
        }
        if (doC) {
          __syncwarp();
          for (int es = lane; es < a.nE; es += 32) {
            uint32_t c = S.cnt[warp * a.nE + es];
            S.cnt[warp * a.nE + es] = 0;
            if ((int)c > a.cmax) { atomicOr(a.status, ST_CNT_OVERFLOW); c = a.cmax; }
            atomicAdd(&a.cnt_core[((uint64_t)cs * a.nE + es) * (a.cmax + 1) + c], 1ull);
          }
          __syncwarp();
        }
      } else if (a.mode == 1) {
        for_each_candidate(a, S.rowtab, cp, self, lane,
                           [&](bool, uint32_t, float, bool inball, uint32_t, bool) { inb += inball; });
        uint32_t tot = inb;
        for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
        if (lane == 0) a.pair_count[ci] = tot;
      } else {
        // mode 2: counting sort of the ball by category into the pair list
        int* hist = S.hist + warp * H;
        for_each_candidate(a, S.rowtab, cp, self, lane, [&](bool, uint32_t, float d2, bool inball, uint32_t, bool) {
          if (inball)
            atomicAdd(&hist[a.lut_one ? category_one(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T)
                                      : category_lut(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T, H)], 1);
        });
        __syncwarp();
        int run = 0;
        for (int h0 = 0; h0 < H; h0 += 32) {
          const int h = h0 + lane;
          const int v = (h < H) ? hist[h] : 0;
          int inc = v;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
          }
          if (h < H) hist[h] = run + inc - v;
          run += __shfl_sync(FULL, inc, 31);
        }
        __syncwarp();
        const unsigned long long off = a.pair_off[ci];
        const unsigned long long lim = a.pair_off[ci + 1];
        for_each_candidate(a, S.rowtab, cp, self, lane, [&](bool, uint32_t slot, float d2, bool inball, uint32_t, bool) {
          if (inball) {
            const int cat = a.lut_one ? category_one(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T)
                                      : category_lut(d2, S.lut, a.lut_n, a.lut_base, a.lut_shift, S.T, H);
            const unsigned long long at = off + (unsigned long long)atomicAdd(&hist[cat], 1);
            if (at < lim && at - a.pair_base < a.pair_cap) {
              a.pair_slot[at - a.pair_base] = slot;
              a.pair_cat[at - a.pair_base] = (uint16_t)cat;
            }
            else atomicOr(a.status, ST_LIST_OVERFLOW);
            ++inb;
          }
        });
        __syncwarp();
        for (int h = lane; h < H; h += 32) hist[h] = 0;
        __syncwarp();
      }
      pairs_lane += inb;
      if (lane == 0) ++centres;
      if (a.rdf_in_smem && doR) {
        // Exchange-based flush keeps every shared bin below 2^32: each time
        // the block's pair count crosses a multiple of 2^30 the warp that
        // crossed it moves all bins to the global uint64 core.
        uint32_t tot = inb;
        for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
        unsigned long long old = 0;
        if (lane == 0) old = atomicAdd(S.since_flush, (unsigned long long)tot);
        old = __shfl_sync(FULL, old, 0);
        if (old / FLUSH != (old + tot) / FLUSH) {
          for (int i = lane; i < a.nC * a.nE * H; i += 32) {
            const uint32_t v = atomicExch(&S.rdf[i], 0u);
            if (v) atomicAdd(&a.rdf_core[i], (unsigned long long)v);
          }
        }
      }
    }
    }
    __syncthreads();
  }
  for (int o = 16; o; o >>= 1) pairs_lane += __shfl_xor_sync(FULL, pairs_lane, o);
  for (int o = 16; o; o >>= 1) tests_lane += __shfl_xor_sync(FULL, tests_lane, o);
  if (lane == 0) {
    atomicAdd(&a.counters[0], pairs_lane);
    atomicAdd(&a.counters[1], centres);
    if (a.tests && a.mode == 0) atomicAdd(a.tests, tests_lane);
  }
  __syncthreads();
  if (a.rdf_in_smem && doR) {
    for (int i = threadIdx.x; i < a.nC * a.nE * H; i += blockDim.x) {
      const uint32_t v = S.rdf[i];
      if (v) atomicAdd(&a.rdf_core[i], (unsigned long long)v);
    }
  }
}

// ------------------------------------------------ merged multi-query pass
// Hull-distance bits of a merged pass: for the queries whose R' = max(R,
// SurfaceCellsCarvingRadius) gave `surf`, bit bits[j] of cmask is set where
// surf >= R2[j] -- the centre test of each query alone
// (src/PARAPROBE_SolverHdl.cpp:3847-3859), from the same ion2surf values.
__global__ void k_cmask_or(const float* __restrict__ surf, uint64_t n, const float* __restrict__ R2,
                           const uint32_t* __restrict__ bits, int nb, uint32_t* __restrict__ cmask) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float v = surf[i];
    uint32_t m = 0;
    for (int j = 0; j < nb; ++j) m |= (v >= R2[j]) ? bits[j] : 0u;
    cmask[i] |= m;
  }
}

__global__ void k_multi_flags(const uint8_t* __restrict__ labels, const uint32_t* __restrict__ cmask,
                              const uint32_t* __restrict__ q_of_type, uint64_t n, uint32_t* __restrict__ flags) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= n; i += (uint64_t)gridDim.x * blockDim.x)
    flags[i] = (i < n && (cmask[i] & q_of_type[labels[i]]) != 0u) ? 1u : 0u;
}

__global__ void k_multi_write(const uint8_t* __restrict__ labels, const uint32_t* __restrict__ cmask,
                              const uint32_t* __restrict__ q_of_type, uint64_t n, const uint32_t* __restrict__ pos,
                              uint32_t* __restrict__ out, uint32_t* __restrict__ count) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if ((cmask[i] & q_of_type[labels[i]]) != 0u) out[pos[i]] = (uint32_t)i;
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = pos[n];
}

// One warp per centre.  The centre's queries are those with a task targeting
// its type whose hull-distance test it passes; its tasks, the tasks of those
// queries that target its type.  The warp walks the candidates within the
// largest radius among its queries once (for_each_candidate_r, nearest rows
// first); a candidate within a query's radius counts as one of that query's
// in-ball pairs whatever its type, and adds to a task's RDF bins (category
// from the query's own threshold table) and kNN list when its type is in the
// task's environment -- exactly the per-centre loop of
// compute_generic_spatstat3 (src/PARAPROBE_SolverHdl.cpp:3975-4101) run for
// each query alone.  RDF bins of all tasks are uint32 counters in shared
// memory, moved to the global uint64 cores whenever the block's adds cross a
// multiple of 2^30; kNN lists are one 32-float row per task in the warp's
// shared memory (rank r in lane r), filled by one ballot per 32 candidates.
constexpr int kMultiWarps = 8;

__global__ void __launch_bounds__(kMultiWarps * 32) k_multi(MultiArgs m) {
  extern __shared__ __align__(16) unsigned char smem[];
  const ScanArgs& a = m.s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  unsigned char* sp = smem;
  unsigned long long* since_flush = (unsigned long long*)sp; sp += 16;
  unsigned long long* scnt = (unsigned long long*)sp; sp += kMultiMaxQueries * 2 * 8;
  MultiQuery* sq = (MultiQuery*)sp; sp += ((sizeof(MultiQuery) * kMultiMaxQueries + 15) & ~size_t(15));
  MultiTask* st = (MultiTask*)sp; sp += ((sizeof(MultiTask) * kMultiMaxTasks + 15) & ~size_t(15));
  unsigned long long* stt = (unsigned long long*)sp; sp += 256 * 8;
  unsigned long long* senv = (unsigned long long*)sp; sp += 256 * 8;
  unsigned long long* stq = (unsigned long long*)sp; sp += kMultiMaxQueries * 8;
  uint32_t* sqt = (uint32_t*)sp; sp += 256 * 4;
  uint32_t* wpairs = (uint32_t*)sp; sp += nwarps * kMultiMaxQueries * 4;
  int8_t* rowtab = (int8_t*)sp; sp += ((ROW_TABLE_ENTRIES * 2 + 15) & ~15);
  float* lists = (float*)sp; sp += (size_t)nwarps * m.lists * 32 * 4;
  uint32_t* srdf = (uint32_t*)sp;  // [rdf_words] when binned in shared memory
  const bool rdf_smem = m.rdf_words > 0;
  for (int i = threadIdx.x; i < m.nq; i += blockDim.x) { sq[i] = m.qs[i]; stq[i] = m.t_of_q[i]; }
  for (int i = threadIdx.x; i < m.nt; i += blockDim.x) st[i] = m.ts[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    stt[i] = m.t_of_type[i];
    senv[i] = m.env_of_type[i];
    sqt[i] = m.q_of_type[i];
  }
  for (int i = threadIdx.x; i < kMultiMaxQueries * 2; i += blockDim.x) scnt[i] = 0ull;
  for (int i = threadIdx.x; i < nwarps * kMultiMaxQueries; i += blockDim.x) wpairs[i] = 0u;
  for (int i = threadIdx.x; i < ROW_TABLE_ENTRIES * 2; i += blockDim.x) rowtab[i] = a.rowtab[i];
  for (uint32_t i = threadIdx.x; i < m.rdf_words; i += blockDim.x) srdf[i] = 0u;
  if (threadIdx.x == 0) *since_flush = 0ull;
  __syncthreads();

  uint32_t* wp = wpairs + warp * kMultiMaxQueries;
  float* L = lists + (size_t)warp * m.lists * 32;
  constexpr unsigned long long FLUSH = 1ull << 30;
  __shared__ uint32_t s_tile, s_next;
  const uint32_t T = max(m.tile, 1u);
  const uint32_t ntiles = (m.ncentres + T - 1) / T;
  for (;;) {
    if (threadIdx.x == 0) { s_tile = atomicAdd(m.work, 1u); s_next = 0; }
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint32_t c0 = tile * T, clen = min(T, m.ncentres - c0);
    for (;;) {
      uint32_t kk = 0;
      if (lane == 0) kk = atomicAdd(&s_next, 1u);
      kk = __shfl_sync(FULL, kk, 0);
      if (kk >= clen) break;
      const uint32_t self = m.centres[c0 + kk];
      const float4 cp = a.ions[self];
      const uint32_t ct = (a.labels ? (uint32_t)a.labels[self] : __float_as_uint(cp.w)) & 255u;
      const uint32_t aq = m.cmask[self] & sqt[ct];
      if (!aq) {  // selection guarantees a query; record and skip otherwise
        if (lane == 0) atomicOr(a.status, ST_TYPE_RANGE);
        continue;
      }
      unsigned long long at = 0;
      float R = 0.f, R2 = 0.f, Rm2 = 0.f;
      for (uint32_t b = aq; b; b &= b - 1u) {
        const int q = __ffs(b) - 1;
        at |= stq[q];
        if (sq[q].R > R) { R = sq[q].R; R2 = sq[q].R2; Rm2 = sq[q].Rm2; }
      }
      at &= stt[ct];
      const unsigned long long atk = at & m.knn_tasks;
      const int nl = __popcll(atk);
      if (nl > m.lists) {  // the host sizes the rows; record and skip otherwise
        if (lane == 0) atomicOr(a.status, ST_BAD_SLOT);
        continue;
      }
      for (int e = lane; e < nl * 32; e += 32) L[e] = kInf();
      __syncwarp();
      uint32_t inb = 0;
      for_each_candidate_r(a, rowtab, cp, self, lane, R, Rm2, R2,
                           [&](bool, uint32_t, float d2, bool inball, uint32_t mt, bool) {
        // in-ball pairs of every query of the centre, whatever the type
        for (uint32_t b = aq; b; b &= b - 1u) {
          const int q = __ffs(b) - 1;
          const uint32_t c = __popc(__ballot_sync(FULL, inball && d2 <= sq[q].R2));
          if (lane == 0) wp[q] += c;
        }
        const unsigned long long et = inball ? (senv[mt & 255u] & at) : 0ull;
        // RDF / RIPK: this candidate's tasks, lane by lane
        for (unsigned long long er = et & m.rdf_tasks; er; er &= er - 1ull) {
          const int t = __ffsll((long long)er) - 1;
          const MultiQuery& Q = sq[st[t].q];
          if (d2 <= Q.R2) {
            const int cat = category_lut(d2, m.lut + Q.lut_off, Q.lut_n, Q.lut_base, Q.lut_shift, m.T + Q.T_off, Q.H);
            ++inb;
            if (rdf_smem) atomicAdd(&srdf[st[t].rdf + cat], 1u);
            else atomicAdd(&m.rdf_core[st[t].rdf + cat], 1ull);
          }
        }
        // kNN: one list row per task of the centre, warp-uniform
        int row = 0;
        for (unsigned long long tb = atk; tb; tb &= tb - 1ull, ++row) {
          const int t = __ffsll((long long)tb) - 1;
          const MultiQuery& Q = sq[st[t].q];
          float* lp = L + row * 32;
          const bool want = ((et >> t) & 1ull) && d2 <= Q.R2;
          uint32_t mask = __ballot_sync(FULL, want && d2 < lp[Q.kmax - 1]);
          while (mask) {
            const int srcl = __ffs(mask) - 1;
            const float x = __shfl_sync(FULL, d2, srcl);
            float v[1] = {lp[lane]};
            list_insert<1>(v, x, lane);
            __syncwarp();
            lp[lane] = v[0];
            __syncwarp();
            mask &= ~(1u << srcl);
            mask &= __ballot_sync(FULL, want && d2 < lp[Q.kmax - 1]);
          }
        }
      });
      // the k-th smallest d^2 of each kNN task -> its bin (or the miss bin)
      int row = 0;
      for (unsigned long long tb = atk; tb; tb &= tb - 1ull, ++row) {
        const int t = __ffsll((long long)tb) - 1;
        const MultiQuery& Q = sq[st[t].q];
        for (int k2 = lane; k2 < Q.nkI; k2 += 32) {
          const int kv = m.kvals[Q.kv_off + k2];
          const float v = L[row * 32 + kv - 1];
          const int cat = (v == kInf()) ? Q.cat_miss
                                        : category_lut(v, m.lut + Q.lut_off, Q.lut_n, Q.lut_base, Q.lut_shift,
                                                       m.T + Q.T_off, Q.H);
          if (cat >= 0) atomicAdd(&m.knn_core[st[t].knn + (uint64_t)k2 * Q.H + cat], 1ull);
        }
      }
      __syncwarp();
      if (lane == 0) {
        for (uint32_t b = aq; b; b &= b - 1u) {
          const int q = __ffs(b) - 1;
          atomicAdd(&scnt[2 * q], (unsigned long long)wp[q]);
          atomicAdd(&scnt[2 * q + 1], 1ull);
          wp[q] = 0u;
        }
      }
      __syncwarp();
      if (rdf_smem) {
        // keep every shared counter below 2^32: when the block's adds cross a
        // multiple of 2^30 the warp that crossed it moves all bins out
        uint32_t tot = inb;
        for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
        unsigned long long old = 0;
        if (lane == 0) old = atomicAdd(since_flush, (unsigned long long)tot);
        old = __shfl_sync(FULL, old, 0);
        if (old / FLUSH != (old + tot) / FLUSH) {
          for (uint32_t i = lane; i < m.rdf_words; i += 32) {
            const uint32_t v = atomicExch(&srdf[i], 0u);
            if (v) atomicAdd(&m.rdf_core[i], (unsigned long long)v);
          }
        }
      }
    }
    __syncthreads();
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < m.rdf_words; i += blockDim.x) {
    const uint32_t v = srdf[i];
    if (v) atomicAdd(&m.rdf_core[i], (unsigned long long)v);
  }
  for (int i = threadIdx.x; i < 2 * m.nq; i += blockDim.x)
    if (scnt[i]) atomicAdd(&m.counters[i], scnt[i]);
}

// ------------------------------------------------- statistics after clustering
// Guard zone about the clusters (clustertask::flag2exclude_guard,
// src/PARAPROBE_SolverHdl.cpp:4790-4817): every ion that is not clustered and
// lies within R (float d^2 <= R^2) of a clustered ion.  One warp per slot;
// warps of unclustered slots move on at once.
__global__ void __launch_bounds__(256) k_guard(ScanArgs a, const uint8_t* __restrict__ clus, uint8_t* guard,
                                               uint64_t n) {
  const int lane = threadIdx.x & 31;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t self = gw; self < n; self += nw) {
    if (!clus[self]) continue;
    const float4 cp = a.ions[self];
    for_each_candidate(a, a.rowtab, cp, (uint32_t)self, lane,
                       [&](bool, uint32_t slot, float, bool inball, uint32_t, bool) {
                         if (inball && !clus[slot]) guard[slot] = 1;
                       });
  }
}

// Neighbours within R of every ion (j != i, float d^2 <= R^2), stored by input
// index: the length of the result list the reference's guard loop takes for a
// clustered ion (src/PARAPROBE_SolverHdl.cpp:4808-4811).  One warp per slot.
__global__ void __launch_bounds__(256) k_ball_count(ScanArgs a, const uint32_t* __restrict__ id_of_slot, uint64_t n,
                                                    uint32_t* __restrict__ count_by_id) {
  const int lane = threadIdx.x & 31;
  const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t self = gw; self < n; self += nw) {
    const float4 cp = a.ions[self];
    uint32_t c = 0;
    for_each_candidate(a, a.rowtab, cp, (uint32_t)self, lane,
                       [&](bool, uint32_t, float, bool inball, uint32_t, bool) { c += inball ? 1u : 0u; });
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(FULL, c, o);
    if (lane == 0) count_by_id[id_of_slot[self]] = c;
  }
}

// labels of the statistics after clustering, in place over the guard flags:
// 1 = neither clustered nor guard (centres and environment), 2 = guard
// (environment only), 3 = clustered (neither)
__global__ void k_cluster_labels(const uint8_t* __restrict__ clus, uint64_t n, uint8_t* guard_then_label) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    guard_then_label[i] = clus[i] ? 3 : (guard_then_label[i] ? 2 : 1);
}

// ------------------------------------------------------- n-point correlations
// One warp per centre (the pass's centre list).  For each environment set of
// the centre type a shared list keeps the K smallest (d^2, ion id) keys with
// their slots; afterwards every task whose targets hold the centre type bins
// the difference vector (neighbour minus centre) of its set's K-th member as
// npc3d::add does (src/PARAPROBE_NPointCorrelations3D.cpp:146-176): skipped
// beyond SpatStatRadiusMax, each component times the float reciprocal of the
// bin width, rounded half away from zero in double, offset by the half edge.
__global__ void __launch_bounds__(256) k_npcorr(ScanArgs a, NpcArgs p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int K = p.K;
  unsigned long long* keysA = (unsigned long long*)smem;                 // [nwarps][emax][32]
  uint32_t* slotsA = (uint32_t*)(keysA + (size_t)nwarps * a.emax * 32);   // [nwarps][emax][32]
  uint32_t* env = slotsA + (size_t)nwarps * a.emax * 32;                  // [nC][256]
  int8_t* rowtab = (int8_t*)(env + a.nC * 256);
  int8_t* scs = rowtab + ROW_TABLE_ENTRIES * 2;                           // 256
  for (int i = threadIdx.x; i < a.nC * 256; i += blockDim.x) env[i] = a.envbits[i];
  for (int i = threadIdx.x; i < ROW_TABLE_ENTRIES * 2; i += blockDim.x) rowtab[i] = a.rowtab[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) scs[i] = a.cslot_of[i];
  __syncthreads();
  unsigned long long* keys = keysA + (size_t)warp * a.emax * 32;
  uint32_t* slots = slotsA + (size_t)warp * a.emax * 32;
  const unsigned long long NONE = ~0ull;
  const uint64_t nxy = (uint64_t)p.edge * p.edge, nxyz = nxy * p.edge;
  for (uint32_t ci = blockIdx.x * nwarps + warp; ci < a.ncentres; ci += gridDim.x * nwarps) {
    const uint32_t self = a.centres[ci];
    const float4 cp = a.ions[self];
    const uint32_t ct = a.labels ? (uint32_t)a.labels[self] : __float_as_uint(cp.w);
    const int cs = scs[ct & 255];
    if (cs < 0 || p.ntk[cs] == 0) continue;
    const int nset = a.nsets[cs];
    for (int e = lane; e < nset * 32; e += 32) { keys[e] = NONE; slots[e] = 0; }
    __syncwarp();
    for_each_candidate(a, rowtab, cp, self, lane,
                       [&](bool valid, uint32_t slot, float d2, bool inball, uint32_t m, bool) {
      (void)valid;
      const uint32_t eb = inball ? env[cs * 256 + (m & 255)] : 0u;
      const unsigned long long key =
          eb ? (((unsigned long long)__float_as_uint(d2) << 32) | p.id_of_slot[slot]) : NONE;
      for (int q = 0; q < nset; ++q) {
        uint32_t mask = __ballot_sync(FULL, ((eb >> q) & 1u) && key < keys[q * 32 + K - 1]);
        while (mask) {
          const int src = __ffs(mask) - 1;
          const unsigned long long x = __shfl_sync(FULL, key, src);
          const uint32_t xs = __shfl_sync(FULL, slot, src);
          unsigned long long* lk = keys + q * 32;
          uint32_t* ls = slots + q * 32;
          const unsigned long long v = lane < K ? lk[lane] : NONE;
          const uint32_t vs = lane < K ? ls[lane] : 0u;
          const int at = __popc(__ballot_sync(FULL, lane < K && v <= x));
          const unsigned long long up = __shfl_up_sync(FULL, v, 1);
          const uint32_t ups = __shfl_up_sync(FULL, vs, 1);
          __syncwarp();
          if (lane < K && lane >= at) {
            lk[lane] = (lane == at) ? x : up;
            ls[lane] = (lane == at) ? xs : ups;
          }
          __syncwarp();
          mask &= ~(1u << src);
          mask &= __ballot_sync(FULL, ((eb >> q) & 1u) && key < keys[q * 32 + K - 1]);
        }
      }
    });
    __syncwarp();
    for (int i = lane; i < p.ntk[cs]; i += 32) {
      const int t = p.tk_task[cs * 32 + i], q = p.tk_set[cs * 32 + i];
      if (keys[q * 32 + K - 1] == NONE) continue;
      const float4 nb = a.ions[slots[q * 32 + K - 1]];
      const float c[3] = {__fsub_rn(nb.x, cp.x), __fsub_rn(nb.y, cp.y), __fsub_rn(nb.z, cp.z)};
      const float d = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(c[0], c[0]), __fmul_rn(c[1], c[1])), __fmul_rn(c[2], c[2])));
      if (!(d <= p.rmax)) continue;
      int64_t b[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float there = __fmul_rn(c[k], p.inv_w);
        const int disc = (there >= 0.f) ? (int)__dadd_rn((double)there, 0.5) : (int)__dsub_rn((double)there, 0.5);
        b[k] = (int64_t)disc + p.half;
      }
      if (b[0] < 0 || b[1] < 0 || b[2] < 0 || b[0] >= p.edge || b[1] >= p.edge || b[2] >= p.edge) {
        atomicOr(a.status, ST_BAD_SLOT);
        continue;
      }
      atomicAdd(&p.counts[(uint64_t)t * nxyz + (uint64_t)b[0] + (uint64_t)b[1] * p.edge + (uint64_t)b[2] * nxy], 1u);
    }
    __syncwarp();
  }
}

// -------------------------------------------------------- K3' brick scan
// The same pass as k_scan, organised around bricks: a brick is up to bx
// consecutive cells of one grid row, and a warp takes the centres of a brick
// (up to `bcap` at a time, in slot order) together.  The stencil rows of the
// brick (every row whose cells can hold a point within R of a point of the
// brick, trimmed in x to the brick's reach) are set up once and their ions
// streamed 32 per step; each candidate is then tested against every centre
// of the batch, whose positions sit in shared memory.  Row set-up and
// candidate loads are shared by the batch instead of paid per centre.  The
// pair set, its distances and bins are those of k_scan: same d^2 expression,
// same in-ball test, same symmetric rule (a pair of two centres is taken by
// the lower slot and credited to both).
template <bool KNN>
__global__ void __launch_bounds__(256) k_brick(ScanArgs a) {
  constexpr int NW = 8;
  extern __shared__ __align__(16) unsigned char smem[];
  const int H = a.H;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int K = KNN ? a.kmax : 1, CB = a.bcap;
  unsigned char* sp = smem;
  unsigned long long* since_flush = (unsigned long long*)sp; sp += 16;
  float4* cposA = (float4*)sp; sp += NW * 32 * 16;
  uint32_t* cslA = (uint32_t*)sp; sp += NW * 32 * 4;
  float* sT = (float*)sp; sp += ((H + 3) & ~3) * 4;
  uint16_t* slut = (uint16_t*)sp; sp += ((a.lut_n + 7) & ~7) * 2;
  uint32_t* srdf = (uint32_t*)sp; sp += (a.rdf_in_smem ? (size_t)a.nC * a.nE * H * 4 : 0);
  float* lists = (float*)sp; sp += (KNN ? (size_t)NW * a.emax * CB * K * 4 : 0);
  int8_t* rowtab = (int8_t*)sp; sp += ROW_TABLE_ENTRIES * 2;
  int8_t* scs = (int8_t*)sp; sp += 256;
  int8_t* ses = (int8_t*)sp; sp += 256;
  int8_t* cctA = (int8_t*)sp; sp += NW * 32;
  int8_t* cesA = (int8_t*)sp; sp += NW * 32;
  int8_t* sidx = (int8_t*)sp;  // [nC][256] (KNN)
  for (int i = threadIdx.x; i < H; i += blockDim.x) sT[i] = a.cat_T[i];
  for (int i = threadIdx.x; i < a.lut_n; i += blockDim.x) slut[i] = a.cat_lut[i];
  for (int i = threadIdx.x; i < ROW_TABLE_ENTRIES * 2; i += blockDim.x) rowtab[i] = a.rowtab[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) { scs[i] = a.cslot_of[i]; ses[i] = a.eslot_of[i]; }
  if (KNN) for (int i = threadIdx.x; i < a.nC * 256; i += blockDim.x) sidx[i] = a.setidx[i];
  if (a.rdf_in_smem) for (int i = threadIdx.x; i < a.nC * a.nE * H; i += blockDim.x) srdf[i] = 0;
  if (threadIdx.x == 0) *since_flush = 0ull;
  __syncthreads();

  const Grid& g = a.g;
  const bool doR = (a.flags & PP_RDF) != 0;
  const bool doK = KNN;
  float4* cpos = cposA + warp * 32;
  uint32_t* csl = cslA + warp * 32;
  int8_t* cct = cctA + warp * 32;
  int8_t* ces = cesA + warp * 32;
  float* L = lists + (size_t)warp * a.emax * CB * K;   // set p, centre c: L + (p * CB + c) * K
  const uint32_t lt = (1u << lane) - 1u, lemask = (2u << lane) - 1u;
  const float m2 = 2.f * g.margin;
  const float Rp = a.R + g.margin, Rp2 = Rp * Rp;
  // rows |dy| = k can hold a neighbour while (k - 1) h - 2 margin <= R + margin
  const int sr_need = (int)floorf((Rp + m2) * g.inv_h) + 1;
  const int sr = min(ROW_SMAX, sr_need);
  const int nrows = (2 * sr + 1) * (2 * sr + 1);
  const int8_t* tab = rowtab + 2 * row_table_offset(sr);
  if (sr_need > ROW_SMAX && threadIdx.x == 0) atomicOr(a.status, ST_BAD_SLOT);
  const uint32_t nbx = (uint32_t)((g.nx + a.bx - 1) / a.bx);
  unsigned long long pairs_lane = 0, centres = 0, tests_lane = 0;
  constexpr unsigned long long FLUSH = 1ull << 30;
  __shared__ uint32_t s_tile, s_next;
  const uint32_t T = a.tile;
  const uint32_t ntiles = (a.nbricks + T - 1) / T;
  for (;;) {
    if (threadIdx.x == 0) { s_tile = atomicAdd(a.work, 1u); s_next = 0; }
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) break;
    const uint32_t b0 = tile * T, blen = min(T, a.nbricks - b0);
    for (;;) {
      uint32_t kb = 0;
      if (lane == 0) kb = atomicAdd(&s_next, 1u);
      kb = __shfl_sync(FULL, kb, 0);
      if (kb >= blen) break;
      const uint32_t b = (a.sample_stride > 1) ? (b0 + kb) * a.sample_stride : b0 + kb;
      const uint32_t zy = b / nbx;
      const int xb = (int)(b - zy * nbx) * a.bx;
      const int y = (int)(zy % (uint32_t)g.ny), z = (int)(zy / (uint32_t)g.ny);
      const int xe = min(xb + a.bx, g.nx);
      const uint64_t hrow = ((uint64_t)z * g.ny + y) * g.nx;
      const uint32_t s1 = a.cell_start[hrow + xe];
      uint32_t pos = a.cell_start[hrow + xb];
      while (pos < s1) {
        // ---- the next batch: up to CB centres of the brick in slot order
        int mc = 0;
        while (pos < s1 && mc < CB) {
          const uint32_t sl = pos + lane;
          const bool isc = sl < s1 && a.cflag[sl] != 0;
          const uint32_t cm = __ballot_sync(FULL, isc);
          const int room = CB - mc, have = __popc(cm);
          uint32_t takem = cm;
          if (have > room) {
            const int lastl = (int)__fns(cm, 0, room);
            takem = cm & ((2u << lastl) - 1u);
            pos += (uint32_t)lastl + 1u;
          } else {
            pos += 32u;
          }
          if ((takem >> lane) & 1u) {
            const int at = mc + __popc(takem & lt);
            const float4 cp = a.ions[sl];
            cpos[at] = cp;
            csl[at] = sl;
            const uint32_t ct = a.labels ? (uint32_t)a.labels[sl] : __float_as_uint(cp.w);
            cct[at] = scs[ct & 255];
            ces[at] = ses[ct & 255];
          }
          mc += min(have, room);
        }
        __syncwarp();
        if (mc == 0) break;
        if (KNN) {
          for (int e = lane; e < a.emax * CB * K; e += 32) L[e] = kInf();
          __syncwarp();
        }
        uint32_t inb = 0;
        // ---- stencil rows of the brick, nearest first
        for (int r0 = 0; r0 < nrows; r0 += 32) {
          const int r = r0 + lane;
          uint32_t st = 0, len = 0;
          if (r < nrows) {
            const int dy = tab[2 * r], dz = tab[2 * r + 1];
            const int yy = y + dy, zz = z + dz;
            if (yy >= 0 && yy < g.ny && zz >= 0 && zz < g.nz) {
              const float gy = fmaxf(0.f, (float)(abs(dy) - 1) * g.h - m2);
              const float gz = fmaxf(0.f, (float)(abs(dz) - 1) * g.h - m2);
              const float rem = Rp2 - gy * gy - gz * gz;
              if (rem >= 0.f) {
                const float half = sqrtf(rem);
                const int x0 = max(0, (int)floorf(((float)xb * g.h - m2 - half) * g.inv_h));
                const int x1 = min(g.nx - 1, (int)floorf(((float)xe * g.h + m2 + half) * g.inv_h));
                const uint64_t cb = ((uint64_t)zz * g.ny + yy) * g.nx;
                int xs = x0;
                if (a.sym) {
                  // cells before the brick in slot order that hold only centres:
                  // each of their pairs with the brick is taken from their side
                  const bool own = (zz == z && yy == y);
                  if (own || zz < z || (zz == z && yy < y)) {
                    const int xend = own ? min(x1, xb - 1) : x1;
                    if (xend >= x0 && a.nc_pre[cb + xend + 1] == a.nc_pre[cb + x0]) xs = xend + 1;
                  }
                }
                if (xs <= x1) {
                  st = a.cell_start[cb + xs];
                  len = a.cell_start[cb + x1 + 1] - st;
                }
              }
            }
          }
          const uint32_t ne = __ballot_sync(FULL, len > 0);
          const int cnt = __popc(ne);
          if (cnt == 0) continue;
          const int src = (lane < cnt) ? (int)__fns(ne, 0, lane + 1) : 0;
          const uint32_t rst = __shfl_sync(FULL, st, src);
          uint32_t rlen = __shfl_sync(FULL, len, src);
          if (lane >= cnt) rlen = 0;
          uint32_t inc = rlen;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
          }
          const uint32_t exc = inc - rlen;
          const uint32_t total = __shfl_sync(FULL, inc, 31);
          int before = 0;
          for (uint32_t bb = 0; bb < total; bb += 32) {
            const uint32_t bitv = (lane < cnt && rlen > 0 && exc >= bb && exc < bb + 32) ? (1u << (exc - bb)) : 0u;
            const uint32_t smask = __reduce_or_sync(FULL, bitv);
            const int row = before + __popc(smask & lemask) - 1;
            before += __popc(smask);
            const int rowc = row < 0 ? 0 : (row > 31 ? 31 : row);
            const uint32_t rs = __shfl_sync(FULL, rst, rowc);
            const uint32_t rp = __shfl_sync(FULL, exc, rowc);
            const uint32_t t = bb + lane;
            const bool valid = t < total;
            const uint32_t slot = rs + (t - rp);
            float4 q = make_float4(kInf(), kInf(), kInf(), 0.f);
            uint32_t m = 0;
            bool jc = false;
            if (valid) {
              q = __ldg(a.ions + slot);
              m = a.labels ? (uint32_t)a.labels[slot] : __float_as_uint(q.w);
              if (a.sym) jc = a.cflag[slot] != 0;
            }
            const int esj = ses[m & 255];
            tests_lane += valid ? (unsigned long long)mc : 0ull;
            for (int c = 0; c < mc; ++c) {
              const float4 cp = cpos[c];
              const uint32_t isl = csl[c];
              const float d2 = dist2(cp.x, cp.y, cp.z, q.x, q.y, q.z);
              const bool inball = valid && (d2 <= a.R2) && (slot != isl) && !(jc && slot < isl);
              const int cs = cct[c];
              if (inball) {
                ++inb;
                int cat = -1;
                if (doR && esj >= 0) {
                  cat = category_lut(d2, slut, a.lut_n, a.lut_base, a.lut_shift, sT, H);
                  const uint32_t idx = ((uint32_t)cs * a.nE + esj) * H + cat;
                  if (a.rdf_in_smem) atomicAdd(&srdf[idx], 1u);
                  else atomicAdd(&a.rdf_core[idx], 1ull);
                }
                if (jc && slot > isl) {
                  // the same pair seen from neighbour j, a centre too
                  ++inb;
                  const int csj = scs[m & 255], esi = ces[c];
                  if (doR && esi >= 0 && csj >= 0) {
                    if (cat < 0) cat = category_lut(d2, slut, a.lut_n, a.lut_base, a.lut_shift, sT, H);
                    const uint32_t idx = ((uint32_t)csj * a.nE + esi) * H + cat;
                    if (a.rdf_in_smem) atomicAdd(&srdf[idx], 1u);
                    else atomicAdd(&a.rdf_core[idx], 1ull);
                  }
                }
              }
              if (KNN && doK) {
                // sorted lists of the K smallest d^2 per (set, centre), one
                // insertion at a time while some lane beats its list's k-th
                const int ps = inball ? (int)sidx[cs * 256 + (m & 255)] : -1;
                uint32_t mask = __ballot_sync(FULL, ps >= 0 && d2 < L[((ps < 0 ? 0 : ps) * CB + c) * K + K - 1]);
                while (mask) {
                  const int srcl = __ffs(mask) - 1;
                  const float x = __shfl_sync(FULL, d2, srcl);
                  const int pp = __shfl_sync(FULL, ps, srcl);
                  float* lp = L + (pp * CB + c) * K;
                  const float v = lane < K ? lp[lane] : kInf();
                  const int at = __popc(__ballot_sync(FULL, lane < K && v <= x));
                  const float up = __shfl_up_sync(FULL, v, 1);
                  __syncwarp();
                  if (lane < K && lane >= at) lp[lane] = (lane == at) ? x : up;
                  __syncwarp();
                  mask &= ~(1u << srcl);
                  mask &= __ballot_sync(FULL, ps >= 0 && d2 < L[((ps < 0 ? 0 : ps) * CB + c) * K + K - 1]);
                }
              }
            }
          }
        }
        // ---- the batch's kNN bins
        if (KNN && doK) {
          __syncwarp();
          for (int c = 0; c < mc; ++c) {
            const int cs = cct[c];
            const int ntg = a.nsets[cs] * a.nkI;
            for (int t = lane; t < ntg; t += 32) {
              const int pp = t / a.nkI, kk = t - pp * a.nkI;
              const float v = L[(pp * CB + c) * K + a.kvals[kk] - 1];
              const int cat = (v == kInf()) ? a.cat_miss
                                            : category_lut(v, slut, a.lut_n, a.lut_base, a.lut_shift, sT, H);
              const int Sg = a.set_list[cs * 32 + pp];
              if (cat >= 0) atomicAdd(&a.knn_core[(((uint64_t)cs * a.nS + Sg) * a.nkI + kk) * H + cat], 1ull);
            }
          }
          __syncwarp();
        }
        pairs_lane += inb;
        if (lane == 0) centres += (unsigned long long)mc;
        if (a.rdf_in_smem && doR) {
          uint32_t tot = inb;
          for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
          unsigned long long old = 0;
          if (lane == 0) old = atomicAdd(since_flush, (unsigned long long)tot);
          old = __shfl_sync(FULL, old, 0);
          if (old / FLUSH != (old + tot) / FLUSH) {
            for (int i = lane; i < a.nC * a.nE * H; i += 32) {
              const uint32_t v = atomicExch(&srdf[i], 0u);
              if (v) atomicAdd(&a.rdf_core[i], (unsigned long long)v);
            }
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
  }
  for (int o = 16; o; o >>= 1) pairs_lane += __shfl_xor_sync(FULL, pairs_lane, o);
  for (int o = 16; o; o >>= 1) tests_lane += __shfl_xor_sync(FULL, tests_lane, o);
  if (lane == 0) {
    atomicAdd(&a.counters[0], pairs_lane);
    atomicAdd(&a.counters[1], centres);
    if (a.tests) atomicAdd(a.tests, tests_lane);
  }
  __syncthreads();
  if (a.rdf_in_smem && doR) {
    for (int i = threadIdx.x; i < a.nC * a.nE * H; i += blockDim.x) {
      const uint32_t v = srdf[i];
      if (v) atomicAdd(&a.rdf_core[i], (unsigned long long)v);
    }
  }
}

// Ion range [st, st + len) of row r of the stencil of the cell block
// [xb, xe) x [yb, ye) x [zb, ze): rows are (yy, zz) with yy in [yb - sr,
// ye - 1 + sr] and zz in [zb - sr, ze - 1 + sr], row r at (yb - sr + ry,
// zb - sr + rz) for (ry, rz) = a.brows[r] (nearest to the block first), each
// trimmed in x to the block's reach and to the reach of the batch's centre
// box [box[0], box[1]] (world coordinates; rows and cells beyond R of the box
// hold no neighbour of these centres); len = 0 when the row cannot hold a
// neighbour of a point of the block.  In symmetric mode the
// leading cells that precede the block's first cell in slot order and hold
// only centres are dropped: their pairs with the block are taken from their
// side (every ion of such a cell has a lower slot than every block centre).
__device__ __forceinline__ void block_row_range(const ScanArgs& a, int r, int nrows, int sr, int xb, int xe, int yb,
                                                int ye, int zb, int ze, bool sym, const float4* box,
                                                uint32_t& st, uint32_t& len) {
  const Grid& g = a.g;
  st = 0;
  len = 0;
  if (r >= nrows) return;
  const int ry = a.brows[2 * r], rz = a.brows[2 * r + 1];
  const int yy = yb - sr + ry, zz = zb - sr + rz;
  if (yy < 0 || yy >= g.ny || zz < 0 || zz >= g.nz) return;
  const float m2 = 2.f * g.margin;
  const float Rp = a.R + g.margin, Rp2 = Rp * Rp;
  const int cy = yy < yb ? yb - yy : (yy >= ye ? yy - (ye - 1) : 0);
  const int cz = zz < zb ? zb - zz : (zz >= ze ? zz - (ze - 1) : 0);
  const float gy = fmaxf(0.f, (float)(cy - 1) * g.h - m2);
  const float gz = fmaxf(0.f, (float)(cz - 1) * g.h - m2);
  const float rem = Rp2 - gy * gy - gz * gz;
  if (rem < 0.f) return;
  const float half = sqrtf(rem);
  int x0 = max(0, (int)floorf(((float)xb * g.h - m2 - half) * g.inv_h));
  int x1 = min(g.nx - 1, (int)floorf(((float)xe * g.h + m2 + half) * g.inv_h));
  {
    // the same against the centre box: the row's ions lie within margin of
    // its cells [lo + c h, lo + (c + 1) h]
    const float4 lo = box[0], hi = box[1];
    const float ry0 = g.loy + (float)yy * g.h, rz0 = g.loz + (float)zz * g.h;
    const float by = fmaxf(0.f, fmaxf(lo.y - (ry0 + g.h), ry0 - hi.y) - m2);
    const float bz = fmaxf(0.f, fmaxf(lo.z - (rz0 + g.h), rz0 - hi.z) - m2);
    const float brem = Rp2 - by * by - bz * bz;
    if (brem < 0.f) return;
    const float bhalf = sqrtf(brem);
    x0 = max(x0, (int)floorf((lo.x - g.lox - m2 - bhalf) * g.inv_h));
    x1 = min(x1, (int)floorf((hi.x - g.lox + m2 + bhalf) * g.inv_h));
    if (x1 < x0) return;
  }
  const uint64_t cb = ((uint64_t)zz * g.ny + yy) * g.nx;
  int xs = x0;
  if (sym) {
    const bool own = (zz == zb && yy == yb);
    if (own || zz < zb || (zz == zb && yy < yb)) {
      const int xend = own ? min(x1, xb - 1) : x1;
      if (xend >= x0 && a.nc_pre[cb + xend + 1] == a.nc_pre[cb + x0]) xs = xend + 1;
    }
  }
  if (xs <= x1) {
    st = a.cell_start[cb + xs];
    len = a.cell_start[cb + x1 + 1] - st;
  }
}

// ----------------------------------------------- K3'' centre-per-lane blocks
// Passes with one centre per lane.  A warp takes up to 32 centres of a block
// of bx x by x bz cells (rows of the block in slot order) and streams the
// block's stencil rows through a per-warp staging buffer, 32 ions at a time;
// every lane then tests the 32 staged ions against its own centre and keeps a
// 32-bit mask of the ions it takes.  A test is half a broadcast shared load,
// the exact d^2 and a predicated bit set -- no branch and no store.  The
// staged ions are stored in pairs, (x0, x1, y0, y1) (z0, z1, w0, w1), so that
// one 128-bit load gives the coordinates of two ions as register pairs and
// the packed f32x2 instructions take their differences and squares two at a
// time (dist2_x2; staged_ion() reads one ion back); the row
// mapping, the record load and the type lookups are paid once per staged ion,
// not once per (centre, ion).  A compact block (cells of R/4 or so, a few
// cells a side) keeps the staged region close to the union of the centres'
// balls.  The pair set and d^2 expression are those of k_scan; what is done
// with the taken pairs is up to the pass (k_lanes: RDF / RIPK bins,
// k_lanes_knn: kNN lists).  Warps fetch blocks `tile` at a time
// from the global work counter, without block barriers.
//
// Box filter: the cell rows hold, beside the centres' neighbours, every ion
// within reach of any point of the cell block.  Each batch of centres takes
// the bounding box of its live centres (kept in shared memory, sbox); the
// rows and their x-ranges are trimmed to the cells within R of that box, and
// before staging each lane measures its candidate's distance to the box and
// drops it when that exceeds R.  The bound is R^2 (1 + 2^-12): the float d^2
// of a centre and the float box distance each lie within a few ulp of their
// exact values (every operation is correctly rounded and the box distance
// never exceeds a centre's distance), so no ion an exact test would take is
// dropped.  Survivors are packed into the staging buffer in stencil order; a
// batch of tests runs each time 32 have gathered, and once more for the rest
// after the last row.  A survivor that finds the buffer full keeps only its
// slot and is reloaded and staged after the tests, so nothing else stays live
// across them.  On the 20M-ion tip (cells of R/4, 4 x 2 x 2 blocks) this took
// the distance tests per pair from 2.66 to 1.78 (RDF) and from 4.43 to 2.92
// (kNN).  Option ScanArgs::no_box_filter stages every candidate, as an A/B
// switch.
//
// lanes_walk calls, warp-uniformly,
//   stage(slot, q, key, code)  per staged ion (its lane): key and code to stage
//   start(self)                a new batch; self = this lane's centre slot or
//                              0xffffffff; returns the lane's centre position
//                              (at infinity for no centre)
//   accept(j, d2, w)           per test of an in-ball staged ion j whose staged
//                              key is w (inlined into the test loop; a constant
//                              true costs nothing)
//   taken(tm, nin, cxx, cyy, czz)  after each staged batch: tm = the lane's
//                              mask, nin = its in-ball ions (counted when
//                              COUNT), the centre's coordinates as f32x2 pairs
//   finish(live)               after the batch's last staged ions
// In symmetric mode (SYM) a lane takes a staged ion when key > its own slot,
// otherwise (KEYED) when key != its own slot; stage() sets key accordingly.
// Without KEYED the key is free for accept() and the centre itself (d^2 = 0)
// passes the in-ball test: the pass excludes it.  With GATED, accept() alone
// decides whether an ion is taken: it must then imply the in-ball test.
__device__ __forceinline__ float4 staged_ion(const float4* cand, int j) {
  const float* f = (const float*)cand + (j >> 1) * 8 + (j & 1);
  return make_float4(f[0], f[2], f[4], f[6]);
}

template <bool SYM, bool COUNT, bool KEYED, bool GATED, class Stage, class Start, class Accept, class Taken,
          class Finish>
__device__ __forceinline__ unsigned long long lanes_walk(const ScanArgs& a, float4* cand, uint32_t* ccode, float4* sbox,
                                                         Stage stage, Start start, Accept accept, Taken taken,
                                                         Finish finish) {
  const Grid& g = a.g;
  const int lane = threadIdx.x & 31;
  const uint32_t lemask = (2u << lane) - 1u;
  // rows up to sr cells away (in y or z) from the block can hold a neighbour
  // (sr = floor((R + 3 margin) / h) + 1, computed by the host with the row table)
  const int sr = a.bsr;
  const int BX = max(a.bx, 1), BY = max(a.by, 1), BZ = max(a.bz, 1);
  const int nry = BY + 2 * sr, nrows = nry * (BZ + 2 * sr);
  const uint32_t nbx = (uint32_t)((g.nx + BX - 1) / BX), nby = (uint32_t)((g.ny + BY - 1) / BY);
  const float R2 = a.R2;
  const uint32_t WT = max(a.tile, 1u);
  unsigned long long tests = 0;  // (centre, staged ion) distance tests, warp-uniform
  for (;;) {
    uint32_t w0 = 0;
    if (lane == 0) w0 = atomicAdd(a.work, WT);
    w0 = __shfl_sync(FULL, w0, 0);
    if (w0 >= a.nbricks) break;
    const uint32_t wend = min(w0 + WT, a.nbricks);
    for (uint32_t wb = w0; wb < wend; ++wb) {
      const uint32_t b = (a.sample_stride > 1) ? wb * a.sample_stride : wb;
      const uint32_t bz_i = b / (nbx * nby), rest = b - bz_i * (nbx * nby);
      const uint32_t by_i = rest / nbx, bx_i = rest - by_i * nbx;
      const int xb = (int)bx_i * BX, yb = (int)by_i * BY, zb = (int)bz_i * BZ;
      const int xe = min(xb + BX, g.nx), ye = min(yb + BY, g.ny), ze = min(zb + BZ, g.nz);
      const int nseg = (ye - yb) * (ze - zb);
      // centres: the block's row segments [cell_start(row, xb), cell_start(row, xe)) in slot order
      int seg = 0;
      uint32_t pos = 0, s1 = 0;
      {
        const uint64_t hrow = ((uint64_t)zb * g.ny + yb) * g.nx;
        pos = a.cell_start[hrow + xb];
        s1 = a.cell_start[hrow + xe];
      }
      for (;;) {
        // ---- the next batch: lane l takes the l-th next centre of the block
        int mc = 0;
        uint32_t self = 0xffffffffu;
        while (mc < 32) {
          if (pos >= s1) {
            if (++seg >= nseg) break;
            const int sy = yb + seg % (ye - yb), sz = zb + seg / (ye - yb);
            const uint64_t hrow = ((uint64_t)sz * g.ny + sy) * g.nx;
            pos = a.cell_start[hrow + xb];
            s1 = a.cell_start[hrow + xe];
            continue;
          }
          const uint32_t sl = pos + lane;
          const uint32_t cm = __ballot_sync(FULL, sl < s1 && a.cflag[sl] != 0);
          const int room = 32 - mc, have = __popc(cm);
          const uint32_t base = pos;
          uint32_t takem = cm;
          if (have > room) {
            const int lastl = (int)__fns(cm, 0, room);
            takem = cm & ((2u << lastl) - 1u);
            pos += (uint32_t)lastl + 1u;
          } else {
            pos += 32u;
          }
          const int ntake = __popc(takem);
          const int want = lane - mc;
          if (want >= 0 && want < ntake) self = base + (uint32_t)__fns(takem, 0, want + 1);
          mc += ntake;
        }
        if (mc == 0) break;
        const float4 cp = start(self);
        const bool lv = cp.x != kInf();
        const uint32_t live = __ballot_sync(FULL, lv);
        if (live) self = lv ? self : 0xffffffffu;
        const unsigned long long cxx = f2_pack(cp.x, cp.x), cyy = f2_pack(cp.y, cp.y), czz = f2_pack(cp.z, cp.z);
        {
          // the live centres' bounding box (order-preserving keys: min and max
          // are exact), kept in shared memory: sbox[0] low, sbox[1] high corner
          const float blx = o2f(__reduce_min_sync(FULL, f2o(lv ? cp.x : kInf())));
          const float bly = o2f(__reduce_min_sync(FULL, f2o(lv ? cp.y : kInf())));
          const float blz = o2f(__reduce_min_sync(FULL, f2o(lv ? cp.z : kInf())));
          const float bhx = o2f(__reduce_max_sync(FULL, f2o(lv ? cp.x : -kInf())));
          const float bhy = o2f(__reduce_max_sync(FULL, f2o(lv ? cp.y : -kInf())));
          const float bhz = o2f(__reduce_max_sync(FULL, f2o(lv ? cp.z : -kInf())));
          if (lane == 0) {
            sbox[0] = make_float4(blx, bly, blz, 0.f);
            sbox[1] = make_float4(bhx, bhy, bhz, 0.f);
          }
          __syncwarp();
        }
        auto put = [&](uint32_t p, const float4& q, uint32_t key, uint32_t code) {
          float* f = (float*)cand + (p >> 1) * 8 + (p & 1);
          f[0] = q.x;
          f[2] = q.y;
          f[4] = q.z;
          f[6] = __uint_as_float(key);
          ccode[p] = code;
        };
        uint32_t fill = 0;  // staged ions waiting for a batch of tests (warp-uniform)
        // the tests of the first nb staged ions (the rest of the buffer holds ions at infinity)
        auto run_batch = [&](uint32_t nb) {
          if (lane >= nb) put(lane, make_float4(kInf(), kInf(), kInf(), 0.f), 0u, 0u);  // no lane takes these
          __syncwarp();
          tests += (unsigned long long)__popc(live) * nb;
          uint32_t tm = 0, nin = 0;
#pragma unroll
          for (int j = 0; j < 32; j += 2) {
            const float4 c0 = cand[j], c1 = cand[j + 1];
            float d0, d1;
            dist2_x2(cxx, cyy, czz, f2_pack(c0.x, c0.y), f2_pack(c0.z, c0.w), f2_pack(c1.x, c1.y), d0, d1);
            const uint32_t k0 = __float_as_uint(c1.z), k1 = __float_as_uint(c1.w);
            const bool in0 = (d0 <= R2) && (!KEYED || (SYM ? (k0 > self) : (k0 != self)));
            const bool in1 = (d1 <= R2) && (!KEYED || (SYM ? (k1 > self) : (k1 != self)));
            if (COUNT) nin += (in0 ? 1u : 0u) + (in1 ? 1u : 0u);
            tm |= ((GATED || in0) && accept(j, d0, k0)) ? (1u << j) : 0u;
            tm |= ((GATED || in1) && accept(j + 1, d1, k1)) ? (2u << j) : 0u;
          }
          taken(tm, nin, cxx, cyy, czz);
          __syncwarp();
        };
        for (int r0 = 0; r0 < nrows && live; r0 += 32) {
          uint32_t st, len;
          block_row_range(a, r0 + lane, nrows, sr, xb, xe, yb, ye, zb, ze, SYM, sbox, st, len);
          const uint32_t ne = __ballot_sync(FULL, len > 0);
          const int cnt_rows = __popc(ne);
          if (cnt_rows == 0) continue;
          const int src = (lane < cnt_rows) ? (int)__fns(ne, 0, lane + 1) : 0;
          const uint32_t rst = __shfl_sync(FULL, st, src);
          uint32_t rlen = __shfl_sync(FULL, len, src);
          if (lane >= cnt_rows) rlen = 0;
          uint32_t inc = rlen;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
          }
          const uint32_t exc = inc - rlen;
          const uint32_t total = __shfl_sync(FULL, inc, 31);
          int before = 0;
          for (uint32_t bb = 0; bb < total; bb += 32) {
            const uint32_t bitv = (lane < cnt_rows && rlen > 0 && exc >= bb && exc < bb + 32) ? (1u << (exc - bb)) : 0u;
            const uint32_t smask = __reduce_or_sync(FULL, bitv);
            const int row = before + __popc(smask & lemask) - 1;
            before += __popc(smask);
            const int rowc = row < 0 ? 0 : (row > 31 ? 31 : row);
            const uint32_t rs = __shfl_sync(FULL, rst, rowc);
            const uint32_t rp = __shfl_sync(FULL, exc, rowc);
            const uint32_t t = bb + lane;
            bool keep = false;
            uint32_t slot = 0;
            float4 q;
            if (t < total) {
              slot = rs + (t - rp);
              q = __ldg(a.ions + slot);
              const float4 lo = sbox[0], hi = sbox[1];
              const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, q.x), __fsub_rn(q.x, hi.x)), 0.f);
              const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, q.y), __fsub_rn(q.y, hi.y)), 0.f);
              const float gz = fmaxf(fmaxf(__fsub_rn(lo.z, q.z), __fsub_rn(q.z, hi.z)), 0.f);
              const float bd = __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
              keep = a.no_box_filter || bd <= a.box_R2;
            }
            const uint32_t km = __ballot_sync(FULL, keep);
            const uint32_t at = fill + (uint32_t)__popc(km & (lemask >> 1));
            uint32_t over = 0xffffffffu;
            if (keep) {
              if (at < 32u) {
                uint32_t key, code;
                stage(slot, q, key, code);
                put(at, q, key, code);
              } else {
                over = slot;
              }
            }
            fill += (uint32_t)__popc(km);
            if (fill >= 32u) {
              run_batch(32u);
              fill -= 32u;
              const uint32_t om = __ballot_sync(FULL, over != 0xffffffffu);
              if (over != 0xffffffffu) {
                const float4 qo = __ldg(a.ions + over);
                uint32_t key, code;
                stage(over, qo, key, code);
                put((uint32_t)__popc(om & (lemask >> 1)), qo, key, code);
              }
              __syncwarp();
            }
          }
        }
        if (fill > 0u) run_batch(fill);
        finish(live);
        __syncwarp();
      }
    }
  }
  return tests;
}

// RDF / RIPK pass.  After each staged batch every lane lists its taken pairs
// at its offset in the batch's pair list and the lanes take the list 64 at a
// time: d^2 is recomputed, binned and added to the (shared) RDF bins, so the
// bin lookup and the histogram atomics run for in-ball pairs only.  In
// symmetric mode a staged ion carries key = its slot when it is a centre and
// 0xffffffff otherwise, and a pair of two centres is taken by the lower slot
// and credited to both.  SMEM (bins in shared memory, fewer than 2^16 of
// them): the staged ion's code and the lane's centre info hold ready bin
// offsets, 16 bits each -- code: env offset (its env slot * H) | its centre
// base (centre slot * nE * H) << 16; info: centre base | env offset << 16;
// 0xffff for none, 0xfffe for a centre without a slot -- so a pair's bin is
// two additions away from its category.
constexpr int kLanesWarps = 16;  // warps per block of k_lanes

template <bool SYM, bool SMEM>
__global__ void __launch_bounds__(kLanesWarps * 32, 2) k_lanes(ScanArgs a) {
  constexpr int NW = kLanesWarps;
  extern __shared__ __align__(16) unsigned char smem[];
  const int H = a.H;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* sp = smem;
  unsigned long long* since_flush = (unsigned long long*)sp; sp += 16;
  float4* candA = (float4*)sp; sp += NW * 32 * 16;
  float4* cposA = (float4*)sp; sp += NW * 32 * 16;
  float4* boxA = (float4*)sp; sp += NW * 2 * 16;
  uint32_t* ccodeA = (uint32_t*)sp; sp += NW * 32 * 4;
  uint32_t* cinfoA = (uint32_t*)sp; sp += NW * 32 * 4;
  uint16_t* plistA = (uint16_t*)sp; sp += NW * 1024 * 2;
  float* sT = (float*)sp; sp += ((H + 4) & ~3) * 4;  // H thresholds, then +inf
  uint32_t* srdf = (uint32_t*)sp; sp += (SMEM ? (size_t)a.nC * a.nE * H * 4 : 0);
  uint16_t* slut = (uint16_t*)sp; sp += ((a.lut_n + 7) & ~7) * 2;
  int8_t* scs = (int8_t*)sp; sp += 256;
  int8_t* ses = (int8_t*)sp;
  for (int i = threadIdx.x; i <= H; i += blockDim.x) sT[i] = i < H ? a.cat_T[i] : kInf();
  for (int i = threadIdx.x; i < a.lut_n; i += blockDim.x) slut[i] = a.cat_lut[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) { scs[i] = a.cslot_of[i]; ses[i] = a.eslot_of[i]; }
  if (SMEM) for (int i = threadIdx.x; i < a.nC * a.nE * H; i += blockDim.x) srdf[i] = 0;
  if (threadIdx.x == 0) *since_flush = 0ull;
  __syncthreads();

  float4* cand = candA + warp * 32;
  float4* cpos = cposA + warp * 32;        // centre of lane c
  uint32_t* ccode = ccodeA + warp * 32;
  uint32_t* cinfo = cinfoA + warp * 32;    // lane c: centre slot * nE | (env slot + 1) << 16, or SMEM's offsets
  uint16_t* plist = plistA + warp * 1024;  // the staged batch's pairs, (lane << 5) | staged index
  unsigned long long pairs_lane = 0, centres = 0;
  constexpr unsigned long long FLUSH = 1ull << 30;
  uint32_t inb = 0;

  const uint32_t cH = (uint32_t)a.nE * (uint32_t)H;  // bins of one centre slot
  auto stage = [&](uint32_t slot, const float4& q, uint32_t& key, uint32_t& code) {
    const uint32_t m = a.labels ? (uint32_t)a.labels[slot] : __float_as_uint(q.w);
    const bool jc = SYM && a.cflag[slot] != 0;
    key = SYM ? (jc ? slot : 0xffffffffu) : slot;
    const int es = ses[m & 255];
    if constexpr (SMEM) {
      const int cs = scs[m & 255];
      const uint32_t cb = !jc ? 0xffffu : (cs < 0 ? 0xfffeu : (uint32_t)cs * cH);
      code = (es < 0 ? 0xffffu : (uint32_t)es * (uint32_t)H) | (cb << 16);
    } else {
      // (env slot + 1) | (centre slot + 1) << 8 | is-centre << 16
      code = (uint32_t)(es + 1) | (jc ? ((uint32_t)(scs[m & 255] + 1) << 8) | 0x10000u : 0u);
    }
  };
  auto start = [&](uint32_t self) {
    float4 cp = make_float4(kInf(), kInf(), kInf(), 0.f);
    int cs = -1, es = -1;
    if (self != 0xffffffffu) {
      cp = a.ions[self];
      const uint32_t ct = a.labels ? (uint32_t)a.labels[self] : __float_as_uint(cp.w);
      cs = scs[ct & 255];
      es = ses[ct & 255];
      if (cs < 0) {  // selection guarantees a slot; record and drop the centre otherwise
        atomicOr(a.status, ST_TYPE_RANGE);
        cp = make_float4(kInf(), kInf(), kInf(), 0.f);
      }
    }
    cpos[lane] = cp;
    if constexpr (SMEM)
      cinfo[lane] = (uint32_t)(cs < 0 ? 0 : cs) * cH | ((es < 0 ? 0xffffu : (uint32_t)es * (uint32_t)H) << 16);
    else
      cinfo[lane] = (uint32_t)(cs < 0 ? 0 : cs) * (uint32_t)a.nE | ((uint32_t)(es + 1) << 16);
    inb = 0;
    return cp;
  };
  auto bin_pair = [&](uint32_t e) {
    const int c = (int)(e >> 5), j = (int)(e & 31u);
    const float4 p = cpos[c];
    const float4 q = staged_ion(cand, j);
    const float d2 = dist2(p.x, p.y, p.z, q.x, q.y, q.z);
    const uint32_t cj = ccode[j], ci = cinfo[c];
    uint32_t cat;
    if (a.lut_one) {
      cat = (uint32_t)category_one(d2, slut, a.lut_n, a.lut_base, a.lut_shift, sT);
    } else {
      cat = (uint32_t)category_lut(d2, slut, a.lut_n, a.lut_base, a.lut_shift, sT, H);
    }
    if constexpr (SMEM) {
      if ((cj & 0xffffu) != 0xffffu) atomicAdd(&srdf[(ci & 0xffffu) + (cj & 0xffffu) + cat], 1u);
      if (SYM && (cj >> 16) != 0xffffu) {
        // the same pair seen from the staged ion, a centre too
        ++inb;
        if ((cj >> 16) != 0xfffeu && (ci >> 16) != 0xffffu) atomicAdd(&srdf[(cj >> 16) + (ci >> 16) + cat], 1u);
      }
    } else {
      const int esj = (int)(cj & 255u) - 1;
      if (esj >= 0) atomicAdd(&a.rdf_core[((ci & 0xffffu) + (uint32_t)esj) * (uint32_t)H + cat], 1ull);
      if (SYM && (cj & 0x10000u)) {
        ++inb;
        const int csj = (int)((cj >> 8) & 255u) - 1;
        const int esc = (int)(ci >> 16) - 1;
        if (esc >= 0 && csj >= 0)
          atomicAdd(&a.rdf_core[((uint32_t)csj * a.nE + (uint32_t)esc) * (uint32_t)H + cat], 1ull);
      }
    }
  };
  auto taken = [&](uint32_t tm, uint32_t, unsigned long long, unsigned long long, unsigned long long) {
    const uint32_t np = __popc(tm);
    uint32_t ex = np;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(FULL, ex, o);
      if (lane >= o) ex += t;
    }
    const uint32_t E = __shfl_sync(FULL, ex, 31);
    inb += np;
    for (uint32_t at = ex - np; tm; ++at) {
      const int j = __ffs(tm) - 1;
      tm &= tm - 1u;
      plist[at] = (uint16_t)((lane << 5) | j);
    }
    __syncwarp();
    for (uint32_t k = lane; k < E; k += 64) {
      const uint32_t e0 = plist[k];
      const bool two = k + 32 < E;
      const uint32_t e1 = two ? plist[k + 32] : 0u;
      bin_pair(e0);
      if (two) bin_pair(e1);
    }
  };
  auto finish = [&](uint32_t live) {
    pairs_lane += inb;
    if (lane == 0) centres += (unsigned long long)__popc(live);
    if (SMEM) {
      // keep every shared bin below 2^32 (see k_scan)
      uint32_t tot = inb;
      for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(FULL, tot, o);
      unsigned long long old = 0;
      if (lane == 0) old = atomicAdd(since_flush, (unsigned long long)tot);
      old = __shfl_sync(FULL, old, 0);
      if (old / FLUSH != (old + tot) / FLUSH) {
        for (int i = lane; i < a.nC * a.nE * H; i += 32) {
          const uint32_t v = atomicExch(&srdf[i], 0u);
          if (v) atomicAdd(&a.rdf_core[i], (unsigned long long)v);
        }
      }
    }
  };
  auto accept = [](int, float, uint32_t) { return true; };
  const unsigned long long tests =
      lanes_walk<SYM, false, true, false>(a, cand, ccode, boxA + warp * 2, stage, start, accept, taken, finish);
  if (lane == 0 && a.tests) atomicAdd(a.tests, tests);

  for (int o = 16; o; o >>= 1) pairs_lane += __shfl_xor_sync(FULL, pairs_lane, o);
  if (lane == 0) {
    atomicAdd(&a.counters[0], pairs_lane);
    atomicAdd(&a.counters[1], centres);
  }
  __syncthreads();
  if (SMEM) {
    for (int i = threadIdx.x; i < a.nC * a.nE * H; i += blockDim.x) {
      const uint32_t v = srdf[i];
      if (v) atomicAdd(&a.rdf_core[i], (unsigned long long)v);
    }
  }
}

// kNN pass (no RDF in the same pass), every type in at most one environment
// set of each centre type.  Each lane keeps, in shared memory, the K smallest
// d^2 of its centre per environment set, largest first (set p, rank r of lane
// l at [(p * K + K - 1 - r) * 32 + l]: the lanes never share a bank, and the
// K-th value of set p is row p * K).  The lists start at the float just above
// R^2, so beating a list's K-th value implies the in-ball test; one more row
// after the last set holds -inf for the ions in no set of the centre type,
// which therefore never pass (no separate test for them).  Stencil rows come
// nearest to the block first, so the lists fill with near ions and their K-th
// values tighten early.  A staged ion carries its environment set for every
// centre slot (4 bits each, nC <= 8), and a lane takes it only when its d^2
// beats the lane's K-th value of that set -- after the first rows few pairs
// are taken.  Taken ions go into the sorted lists.  At the end of the batch
// the k-th values are binned (a missing neighbour at R + EPSILON), as k_scan
// does.
constexpr int kLanesKnnWarps = 8;

// KB > 0: K <= KB, and an insertion loads the whole list at once (KB
// independent shared loads) instead of walking it; KB = 0: any K.
// UNI: every centre slot maps a type to the same local environment set (the
// usual all-pairs task lists); a staged ion then carries that set's list row
// as a ready offset instead of one 4-bit set index per centre slot.
// CAT: the lists hold bin categories (uint16), not d^2 -- half the shared
// memory, for many sets of large k (8 sets of k = 20 fit two blocks of 8
// warps per SM instead of one).  The k-th smallest category is the category
// of the k-th smallest d^2 (categories rise with d^2), which is all the
// histogram needs.  Each set keeps, beside its categories, the float test
// threshold: the smallest d^2 of its K-th category (just above R^2 while the
// list is not full); an ion beats it exactly when its category is below the
// K-th one, so the test stays one float compare; a taken ion's category is
// looked up once, at insertion, and the binning at the end needs none.
template <int KB, bool UNI, bool CAT>
__global__ void __launch_bounds__(kLanesKnnWarps * 32, 3) k_lanes_knn(ScanArgs a) {
  constexpr int NW = kLanesKnnWarps;
  constexpr uint32_t CNONE = 0xffffu;  // CAT: an empty list place (above every category)
  extern __shared__ __align__(16) unsigned char smem[];
  const int H = a.H, K = a.kmax, EM = a.emax;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // per warp: float rows -- the lists (EM * K rows) or, with CAT, one threshold
  // row per set -- then the row of "no set"; with CAT the category rows after
  const int frows = CAT ? EM + 1 : EM * K + 1;
  unsigned char* sp = smem;
  float4* candA = (float4*)sp; sp += NW * 32 * 16;
  float4* boxA = (float4*)sp; sp += NW * 2 * 16;
  uint32_t* ccodeA = (uint32_t*)sp; sp += NW * 32 * 4;
  float* listA = (float*)sp; sp += (size_t)NW * frows * 32 * 4;
  uint16_t* catA = (uint16_t*)sp; sp += CAT ? (((size_t)NW * EM * K * 32 * 2 + 15) & ~size_t(15)) : 0;
  float* sT = (float*)sp; sp += ((H + 4) & ~3) * 4;  // H thresholds, then +inf
  uint16_t* slut = (uint16_t*)sp; sp += ((a.lut_n + 7) & ~7) * 2;
  int8_t* scs = (int8_t*)sp; sp += 256;
  uint32_t* skey = (uint32_t*)sp;  // [256] per type: its environment set (EM: none) for every centre slot, 4 bits each
  const uint32_t RSTRIDE = CAT ? 32u : (uint32_t)K * 32u;  // float rows between sets
  for (int i = threadIdx.x; i <= H; i += blockDim.x) sT[i] = i < H ? a.cat_T[i] : kInf();
  for (int i = threadIdx.x; i < a.lut_n; i += blockDim.x) slut[i] = a.cat_lut[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    scs[i] = a.cslot_of[i];
    uint32_t key = 0;
    if (UNI) {
      const int si = a.nC > 0 ? a.setidx[i] : -1;
      key = (uint32_t)(si < 0 ? EM : si) * RSTRIDE;
    } else {
      for (int c = 0; c < a.nC; ++c) {
        const int si = a.setidx[c * 256 + i];
        key |= (uint32_t)(si < 0 ? EM : si) << (4 * c);
      }
    }
    skey[i] = key;
  }
  __syncthreads();

  float4* cand = candA + warp * 32;
  uint32_t* ccode = ccodeA + warp * 32;
  // set p, rank r at L[(p * K + K - 1 - r) * 32]; with CAT, set p's threshold
  // at L[p * 32] and its rank r at C[(p * K + K - 1 - r) * 32]
  float* L = listA + (size_t)warp * frows * 32 + lane;
  uint16_t* C = catA + (size_t)warp * EM * K * 32 + lane;
  L[(uint32_t)EM * RSTRIDE] = -kInf();  // the row of "no set": nothing beats it
  const float RUP = (a.R2 >= 0.f && a.R2 < kInf()) ? __uint_as_float(__float_as_uint(a.R2) + 1u) : kInf();
  unsigned long long pairs_lane = 0, centres = 0;
  uint32_t inb = 0;
  int cs = -1, nset = 0, sh = 0;  // centre slot, its sets, 4 * slot (its nibble in a staged key)
  uint32_t me = 0xffffffffu;      // this lane's centre slot

  // the staged key carries the ion's environment set for every centre slot
  // (read by the test loop with the position), the code its slot
  auto stage = [&](uint32_t slot, const float4& q, uint32_t& key, uint32_t& code) {
    const uint32_t m = (a.labels ? (uint32_t)a.labels[slot] : __float_as_uint(q.w)) & 255u;
    key = skey[m];
    code = slot;
  };
  auto start = [&](uint32_t self) {
    float4 cp = make_float4(kInf(), kInf(), kInf(), 0.f);
    cs = -1;
    if (self != 0xffffffffu) {
      cp = a.ions[self];
      const uint32_t ct = a.labels ? (uint32_t)a.labels[self] : __float_as_uint(cp.w);
      cs = scs[ct & 255];
      if (cs < 0) {  // selection guarantees a slot; record and drop the centre otherwise
        atomicOr(a.status, ST_TYPE_RANGE);
        cp = make_float4(kInf(), kInf(), kInf(), 0.f);
      }
    }
    nset = cs >= 0 ? a.nsets[cs] : 0;
    sh = 4 * (cs < 0 ? 0 : cs);
    if constexpr (CAT) {
      for (int p = 0; p < nset; ++p) L[p * 32] = RUP;
      for (int e = 0; e < nset * K; ++e) C[e * 32] = (uint16_t)CNONE;
    } else {
      for (int e = 0; e < nset * K; ++e) L[e * 32] = RUP;
    }
    me = cp.x != kInf() ? self : 0xffffffffu;
    inb = 0;
    return cp;
  };
  // float row (offset) of a staged key's environment set for this lane's centre type
  auto row_of = [&](uint32_t w) -> uint32_t { return UNI ? w : ((w >> sh) & 15u) * RSTRIDE; };
  auto accept = [&](int, float d2, uint32_t w) {
    // the set's K-th value or threshold (the -inf row for ions in no set)
    return d2 < L[row_of(w)];
  };
  auto insert = [&](uint32_t row, float d2) {
    float* Lp = L + row;  // row s holds rank K - 1 - s
    if (!(d2 < Lp[0])) return;
    if constexpr (CAT) {
      int c;
      if (a.lut_one) {
        c = category_one(d2, slut, a.lut_n, a.lut_base, a.lut_shift, sT);
      } else {
        c = category_lut(d2, slut, a.lut_n, a.lut_base, a.lut_shift, sT, H);
      }
      uint16_t* Cp = C + (row / 32u) * (uint32_t)K * 32u;
      if constexpr (KB > 0) {
        int v[KB];
#pragma unroll
        for (int s = 0; s < KB; ++s) v[s] = (s < K) ? (int)Cp[s * 32] : -1;
#pragma unroll
        for (int s = 0; s < KB; ++s)
          if (s < K) v[s] = min(v[s], max(s + 1 < KB ? v[s + 1 < KB ? s + 1 : s] : -1, c));
#pragma unroll
        for (int s = 0; s < KB; ++s)
          if (s < K) Cp[s * 32] = (uint16_t)v[s];
        Lp[0] = (v[0] == (int)CNONE) ? RUP : sT[v[0]];
      } else {
        int r = K - 1;
        while (r > 0) {
          const int v = Cp[(K - r) * 32];  // rank r - 1
          if (!(v > c)) break;
          Cp[(K - 1 - r) * 32] = (uint16_t)v;
          --r;
        }
        Cp[(K - 1 - r) * 32] = (uint16_t)c;
        const int kth = Cp[0];
        Lp[0] = (kth == (int)CNONE) ? RUP : sT[kth];
      }
    } else if constexpr (KB > 0) {
      // the sorted list with d2 in and its largest value out, as a min/max
      // network over ranks: new[r] = min(v[r], max(v[r - 1], d2)), new[0] =
      // min(v[0], d2); rank r - 1 is the next row
      float v[KB];
#pragma unroll
      for (int s = 0; s < KB; ++s) v[s] = (s < K) ? Lp[s * 32] : -kInf();
#pragma unroll
      for (int s = 0; s < KB; ++s)
        if (s < K) Lp[s * 32] = fminf(v[s], fmaxf(s + 1 < KB ? v[s + 1 < KB ? s + 1 : s] : -kInf(), d2));
    } else {
      int r = K - 1;
      while (r > 0) {
        const float v = Lp[(K - r) * 32];  // rank r - 1
        if (!(v > d2)) break;
        Lp[(K - 1 - r) * 32] = v;
        --r;
      }
      Lp[(K - 1 - r) * 32] = d2;
    }
  };
  auto taken = [&](uint32_t tm, uint32_t nin, unsigned long long cxx, unsigned long long cyy, unsigned long long czz) {
    inb += nin;
    float cx, cy, cz, dup;
    f2_unpack(cxx, cx, dup);
    f2_unpack(cyy, cy, dup);
    f2_unpack(czz, cz, dup);
    while (tm) {
      const int j = __ffs(tm) - 1;
      tm &= tm - 1u;
      const float4 q = staged_ion(cand, j);
      const float d2 = dist2(cx, cy, cz, q.x, q.y, q.z);
      if (d2 == 0.f && ccode[j] == me) continue;  // the centre itself
      insert(row_of(__float_as_uint(q.w)), d2);
    }
  };
  auto finish = [&](uint32_t live) {
    if (lane == 0) centres += (unsigned long long)__popc(live);
    // every live centre met itself once in the in-ball count (d^2 = 0)
    pairs_lane += inb - (me != 0xffffffffu ? 1u : 0u);
    // the k-th smallest d^2 (category) of each set -> its bin (or the miss
    // bin); with KB, a set's categories are found first (independent loads)
    // and added after
    for (int p = 0; p < nset; ++p) {
      const int Sg = a.set_list[cs * 32 + p];
      unsigned long long* core = a.knn_core + ((uint64_t)cs * a.nS + Sg) * a.nkI * H;
      auto cat_of = [&](int kk) {
        if constexpr (CAT) {
          const int v = C[(p * K + K - a.kvals[kk]) * 32];
          return (v == (int)CNONE) ? a.cat_miss : v;
        } else {
          const float v = L[(p * K + K - a.kvals[kk]) * 32];
          return (v == RUP) ? a.cat_miss : category_lut(v, slut, a.lut_n, a.lut_base, a.lut_shift, sT, H);
        }
      };
      if constexpr (KB > 0) {
        int cats[KB];
#pragma unroll
        for (int kk = 0; kk < KB; ++kk) cats[kk] = kk < a.nkI ? cat_of(kk) : -1;
#pragma unroll
        for (int kk = 0; kk < KB; ++kk)
          if (cats[kk] >= 0) atomicAdd(&core[(uint64_t)kk * H + cats[kk]], 1ull);
      } else {
        for (int kk = 0; kk < a.nkI; ++kk) {
          const int cat = cat_of(kk);
          if (cat >= 0) atomicAdd(&core[(uint64_t)kk * H + cat], 1ull);
        }
      }
    }
  };
  const unsigned long long tests =
      lanes_walk<false, true, false, true>(a, cand, ccode, boxA + warp * 2, stage, start, accept, taken, finish);
  if (lane == 0 && a.tests) atomicAdd(a.tests, tests);

  for (int o = 16; o; o >>= 1) pairs_lane += __shfl_xor_sync(FULL, pairs_lane, o);
  if (lane == 0) {
    atomicAdd(&a.counters[0], pairs_lane);
    atomicAdd(&a.counters[1], centres);
  }
}

// --------------------------------------------------------------- K5 batched
// One work item = (tile of geometry centres, group of G realisations).  Labels
// and centre masks are stored group-major, G realisations interleaved per slot
// -- realisation g*G + r of slot s at (g * n + s) * G + r -- so one G-byte load
// gives a neighbour's type in every realisation of the group while neighbours
// stay close in memory.  One warp walks one centre's category-sorted pair list
// once for the whole group.  For kNN every list entry knows its rank among the
// members of its environment set met so far, and the entry of rank k-1 is the
// k-th nearest member (the list is ordered by category, which is all a
// histogram of distances resolves).  RDF bins (32-bit) and, when KS, kNN bins
// (16-bit, two per word) of the group live in shared memory, bin-major with G
// counters per bin, and are added to the global cores once per item.  The host
// sizes a tile so that no 16-bit bin can reach 65536 within one item (at most
// one count per centre) and no RDF bin 2^32 (tile x longest list < 2^31).
template <int G>
struct LabelWord;
template <> struct LabelWord<1> { using T = uint8_t; };
template <> struct LabelWord<2> { using T = uint16_t; };
template <> struct LabelWord<4> { using T = uint32_t; };
template <> struct LabelWord<8> { using T = unsigned long long; };

struct ApplyLayout {
  int nrdf, nknn, nkw, nenv, nset8;
  __host__ __device__ ApplyLayout(const ApplyArgs& a, int G, bool ks) {
    const bool knn = (a.flags & PP_MKNN) != 0;
    nrdf = (a.flags & PP_RDF) ? a.nC * a.nE * a.H : 0;
    nknn = (ks && knn) ? a.nC * a.nS * a.nkI * a.H : 0;
    nkw = (nknn * G + 1) / 2;
    nenv = (knn && !a.disjoint) ? a.nC * 256 : 0;
    nset8 = (knn && a.disjoint) ? a.nC * 256 : 0;
  }
  // per-warp set counters live in shared memory only for overlapping sets
  __host__ __device__ int seen_words(int G, int nwarps, int nsmax) const { return nenv ? nwarps * G * nsmax : 0; }
  __host__ __device__ size_t bytes(int G, int nwarps, int nsmax) const {
    return (size_t)16 * G + (size_t)nrdf * G * 4 + (size_t)nkw * 4 + (size_t)seen_words(G, nwarps, nsmax) * 4 +
           (size_t)nenv * 4 + nset8 + 768;
  }
};

template <int G, bool KS>
__global__ void __launch_bounds__(1024, 1) k_apply(ApplyArgs a) {
  using W = typename LabelWord<G>::T;
  extern __shared__ __align__(16) unsigned char smem[];
  const int H = a.H;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const bool knn = (a.flags & PP_MKNN) != 0;
  const ApplyLayout L(a, G, KS);
  const int nsmax = max(a.nsmax, 1);
  unsigned long long* sCnt = (unsigned long long*)smem;      // [G][2] pairs, centres
  uint32_t* sRdf = (uint32_t*)(sCnt + 2 * G);                 // [nrdf][G]
  uint32_t* sKnn = sRdf + L.nrdf * G;                         // [nknn][G] 16-bit
  uint32_t* sSeen = sKnn + L.nkw;                             // [nwarps][G][nsmax]
  uint32_t* sEnv = sSeen + L.seen_words(G, nwarps, nsmax);    // [nC][256] (overlapping sets)
  int8_t* sSet = (int8_t*)(sEnv + L.nenv);                    // [nC][256] (disjoint sets)
  int8_t* sC = sSet + L.nset8;                                // 256
  int8_t* sE = sC + 256;                                      // 256
  int8_t* sK = sE + 256;                                      // 256: k -> index into kvals, -1
  __shared__ uint32_t s_item;
  for (int i = threadIdx.x; i < 2 * G; i += blockDim.x) sCnt[i] = 0;
  for (int i = threadIdx.x; i < L.nrdf * G + L.nkw; i += blockDim.x) sRdf[i] = 0;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) { sC[i] = a.cslot_of[i]; sE[i] = a.eslot_of[i]; sK[i] = -1; }
  for (int i = threadIdx.x; i < L.nenv; i += blockDim.x) sEnv[i] = a.envbits[i];
  for (int i = threadIdx.x; i < L.nset8; i += blockDim.x) sSet[i] = a.setidx[i];
  __syncthreads();
  if (knn)
    for (int i = threadIdx.x; i < a.nkI; i += blockDim.x)
      if (a.kvals[i] >= 1 && a.kvals[i] <= 255) sK[a.kvals[i]] = (int8_t)i;
  __syncthreads();
  uint32_t* seen = sSeen + warp * G * nsmax;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t ntiles = (a.ncentres + a.tile - 1) / a.tile;
  const uint32_t nitems = ntiles * (uint32_t)a.ngroups;
  const uint64_t knn_real = (uint64_t)a.nC * a.nS * a.nkI * H;   // global kNN bins per realisation
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.work, 1u);
    __syncthreads();
    const uint32_t item = s_item;
    __syncthreads();
    if (item >= nitems) break;
    const uint32_t tile = item / a.ngroups, grp = item - tile * a.ngroups;
    const int rb = (int)grp * G;
    const W* lab = (const W*)(a.labels + (uint64_t)grp * a.n * G);
    const W* okw = (const W*)(a.centre_ok + ((uint64_t)grp * a.nc_total + a.cbase) * G);
    const uint32_t c0 = tile * a.tile, c1 = min(c0 + a.tile, a.ncentres);
    // one kNN count: bin (c, set q, order kk, category) of realisation rb + r
    auto knn_add = [&](int c, int q, int kk, int cat, int r) {
      const int Sg = a.set_list[c * 32 + q];
      const uint32_t bin = (((uint32_t)c * a.nS + Sg) * a.nkI + kk) * H + cat;
      if (KS) {
        const uint32_t i16 = bin * G + r;
        atomicAdd(&sKnn[i16 >> 1], 1u << ((i16 & 1u) * 16));
      } else {
        atomicAdd(&a.knn_core[(uint64_t)(a.rbase + rb + r) * knn_real + bin], 1ull);
      }
    };
    for (uint32_t ci = c0 + warp; ci < c1; ci += nwarps) {
      const uint32_t self = a.centres[ci];
      const W lw = lab[self];
      const W ow = okw[ci];
      int cs[G];
      uint32_t cnt[G];   // disjoint sets: lane q counts the members of set q met so far
      uint32_t kn = 0;   // realisations whose kNN walk is still open
      bool any = false;
#pragma unroll
      for (int r = 0; r < G; ++r) {
        const bool ok = ((ow >> (8 * r)) & 0xff) != 0 && rb + r < a.nreal;
        cs[r] = ok ? (int)sC[(lw >> (8 * r)) & 0xff] : -1;
        any |= cs[r] >= 0;
        if (knn && cs[r] >= 0 && a.nsets[cs[r]] > 0) kn |= 1u << r;
        cnt[r] = 0;
        if (L.nenv && lane < nsmax) seen[r * nsmax + lane] = 0;
      }
      if (!any) continue;
      __syncwarp();
      const unsigned long long o0 = a.pair_off[ci], o1 = a.pair_off[ci + 1];
      if (lane == 0) {
#pragma unroll
        for (int r = 0; r < G; ++r)
          if (cs[r] >= 0) { atomicAdd(&sCnt[2 * r], o1 - o0); atomicAdd(&sCnt[2 * r + 1], 1ull); }
      }
      // entries are loaded two steps ahead (category and slot) and one step
      // ahead (the neighbour's labels), so the dependent loads of a step are
      // in flight while the step before it is binned
      int cat_n = 0, cat_nn = 0;
      uint32_t slot_nn = 0;
      W nw_n = 0;
      {
        const unsigned long long e0 = o0 + lane, e1 = o0 + 32 + lane;
        if (e0 < o1) {
          cat_n = a.pair_cat[e0 - a.pair_base];
          nw_n = lab[a.pair_slot[e0 - a.pair_base]];
        }
        if (e1 < o1) {
          cat_nn = a.pair_cat[e1 - a.pair_base];
          slot_nn = a.pair_slot[e1 - a.pair_base];
        }
      }
      for (unsigned long long k0 = o0; k0 < o1; k0 += 32) {
        if (!L.nrdf && !kn) break;
        const unsigned long long e = k0 + lane;
        const bool valid = e < o1;
        const int cat = cat_n;
        const W nw = nw_n;
        // advance the pipeline: labels of the next step, entries of the one after
        cat_n = cat_nn;
        nw_n = (e + 32 < o1) ? lab[slot_nn] : (W)0;
        if (e + 64 < o1) {
          cat_nn = a.pair_cat[e + 64 - a.pair_base];
          slot_nn = a.pair_slot[e + 64 - a.pair_base];
        }
#pragma unroll
        for (int r = 0; r < G; ++r) {
          const int c = cs[r];
          if (c < 0) continue;
          const int t = (int)((nw >> (8 * r)) & 0xff);
          if (L.nrdf && valid) {
            const int es = sE[t];
            if (es >= 0) atomicAdd(&sRdf[(((uint32_t)c * a.nE + es) * H + cat) * G + r], 1u);
          }
          if (!((kn >> r) & 1u)) continue;
          const int nset = a.nsets[c];
          if (a.disjoint) {
            // each type is in at most one set.  One ballot per bit of the set
            // index gives every lane two masks: the lanes holding members of
            // its entry's set, and the lanes holding members of set `lane`
            const int q = valid ? (int)sSet[c * 256 + t] : -1;
            const bool mem = q >= 0;
            const uint32_t m0 = __ballot_sync(FULL, mem);
            if (!m0) continue;
            uint32_t mine = m0, own = m0;
            const int nb = nset > 1 ? 32 - __clz(nset - 1) : 0;
            for (int b = 0; b < nb; ++b) {
              const uint32_t bb = __ballot_sync(FULL, (q >> b) & 1);
              mine &= ((q >> b) & 1) ? bb : ~bb;
              own &= ((lane >> b) & 1) ? bb : ~bb;
            }
            const uint32_t before = __shfl_sync(FULL, cnt[r], q & 31);
            if (mem) {
              const uint32_t rank = before + __popc(mine & lt);   // 0-based among set members
              if (rank < (uint32_t)a.kmax) {
                const int kk = sK[rank + 1];
                if (kk >= 0) knn_add(c, q, kk, cat, r);
              }
            }
            cnt[r] += __popc(own);
            if (!__any_sync(FULL, lane < nset && cnt[r] < (uint32_t)a.kmax)) kn &= ~(1u << r);
            continue;
          }
          uint32_t* sr = seen + r * nsmax;
          const uint32_t eb = valid ? sEnv[c * 256 + t] : 0u;
          bool open = false;
          for (int q = 0; q < nset; ++q) {
            const bool mem = (eb >> q) & 1u;
            const uint32_t m = __ballot_sync(FULL, mem);
            if (!m) { open |= sr[q] < (uint32_t)a.kmax; continue; }
            const uint32_t before = sr[q];
            if (mem) {
              const uint32_t rank = before + __popc(m & lt);
              if (rank < (uint32_t)a.kmax) {
                const int kk = sK[rank + 1];
                if (kk >= 0) knn_add(c, q, kk, cat, r);
              }
            }
            const uint32_t after = before + __popc(m);
            __syncwarp();
            if (lane == 0) sr[q] = after;
            __syncwarp();
            open |= after < (uint32_t)a.kmax;
          }
          if (!open) kn &= ~(1u << r);
        }
      }
      // members not met within R: the remaining orders of each set are misses
#pragma unroll
      for (int r = 0; r < G; ++r) {
        const int c = cs[r];
        if (!knn || c < 0) continue;
        const int nset = a.nsets[c];
        for (int q = 0; q < nset; ++q) {
          uint32_t got = __shfl_sync(FULL, cnt[r], q);
          if (L.nenv) got = seen[r * nsmax + q];
          if (got >= (uint32_t)a.kmax) continue;
          for (int kk = lane; kk < a.nkI; kk += 32)
            if (got < (uint32_t)a.kvals[kk]) knn_add(c, q, kk, a.cat_miss, r);
        }
      }
      __syncwarp();
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * G; i += blockDim.x) {
      const unsigned long long v = sCnt[i];
      if (v) {
        if (a.count) atomicAdd(&a.counters[2 * ((uint64_t)a.rbase + rb) + i], v);
        sCnt[i] = 0;
      }
    }
    for (int i = threadIdx.x; i < L.nrdf * G; i += blockDim.x) {
      const uint32_t v = sRdf[i];
      if (v) {
        const int r = i % G, bin = i / G;
        atomicAdd(&a.rdf_core[(uint64_t)(a.rbase + rb + r) * L.nrdf + bin], (unsigned long long)v);
        sRdf[i] = 0;
      }
    }
    if (KS) {
      for (int w = threadIdx.x; w < L.nkw; w += blockDim.x) {
        const uint32_t v = sKnn[w];
        if (v) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint32_t c16 = (v >> (16 * h)) & 0xffffu;
            if (c16) {
              const uint32_t i16 = 2 * w + h;
              const int r = i16 % G;
              const uint32_t bin = i16 / G;
              atomicAdd(&a.knn_core[(uint64_t)(a.rbase + rb + r) * knn_real + bin], (unsigned long long)c16);
            }
          }
          sKnn[w] = 0;
        }
      }
    }
    __syncthreads();
  }
}

// --------------------------------------------------------- K5 batched kNN
// Walk: one warp per centre, lane r = realisation grp * 32 + r.  All lanes
// read the same pair-list entry (one broadcast load) and their own label of
// the neighbour (32 consecutive bytes), so the walk costs a few instructions
// per entry for 32 realisations.  Each lane counts the members of each set it
// has met; the entry that makes a set's count k is its k-th nearest member
// (the list is in category order).  The walk ends when every lane has k_max
// members of every set, or the list ends (the rest are misses).
template <bool DISJ>
__global__ void __launch_bounds__(512, 2) k_knn_walk(KnnArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int NT = a.nsmax * a.nkI;
  // set table per centre type, plus a last row that matches nothing (lanes
  // that are no centre in their realisation walk it without effect):
  // DISJ: set index of a type (int8, -1 = none); else set bit mask (uint32)
  const int nrow = (a.nC + 1) * 256;
  unsigned char* sTab = smem;
  int* sNs = (int*)(smem + (size_t)nrow * (DISJ ? 1 : 4));     // [nC]
  int8_t* sC = (int8_t*)(sNs + a.nC);                          // 256
  int8_t* sK = sC + 256;                                       // 256
  uint8_t* sCnt = (uint8_t*)(sK + 256);                        // [nwarps][nsmax][32]
  for (int i = threadIdx.x; i < nrow; i += blockDim.x) {
    const bool last = i >= a.nC * 256;
    if (DISJ) ((int8_t*)sTab)[i] = last ? (int8_t)-1 : a.setidx[i];
    else ((uint32_t*)sTab)[i] = last ? 0u : a.envbits[i];
  }
  for (int i = threadIdx.x; i < a.nC; i += blockDim.x) sNs[i] = a.nsets[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) { sC[i] = a.cslot_of[i]; sK[i] = -1; }
  __syncthreads();
  for (int i = threadIdx.x; i < a.nkI; i += blockDim.x)
    if (a.kvals[i] >= 1 && a.kvals[i] <= 255) sK[a.kvals[i]] = (int8_t)i;
  __syncthreads();
  uint8_t* cnt = sCnt + warp * a.nsmax * 32 + lane;
  const uint8_t* lab = a.labels + (uint64_t)a.grp * a.n * 32 + lane;
  const uint8_t* okp = a.centre_ok + (uint64_t)a.grp * a.ncentres * 32 + lane;
  const bool real = a.grp * 32 + lane < a.nreal;
  const int kmax = a.kmax, nkI = a.nkI;
  const uint32_t ntiles = (a.cn + a.tile - 1) / a.tile;
  // each warp fetches its own tile of centres (no block barrier: list
  // lengths differ from centre to centre)
  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(a.work, 1u);
    item = __shfl_sync(FULL, item, 0);
    if (item >= ntiles) break;
    const uint32_t l0 = item * a.tile, l1 = min(l0 + a.tile, a.cn);
    for (uint32_t li = l0; li < l1; ++li) {
      const uint32_t ci = a.c0 + li;
      const uint32_t self = a.centres[ci];
      const bool ok = real && okp[(uint64_t)ci * 32] != 0;
      const int c = ok ? (int)sC[lab[(uint64_t)self * 32]] : -1;
      const int nset = c >= 0 ? sNs[c] : 0;
      int unsat = nset;                   // sets with fewer than k_max members met
      for (int q = 0; q < a.nsmax; ++q) cnt[q * 32] = 0;
      const int row = (c >= 0 ? c : a.nC) * 256;
      const unsigned long long o0 = a.pair_off[ci], o1 = a.pair_off[ci + 1];
      // records of this centre: one 64-byte row per (set, order) slot,
      // realisations along the row; a slot is written when its member is met
      uint16_t* out = a.rec + (uint64_t)li * NT * 32 + lane;
      // 32 entries per coalesced load (one step ahead), then neighbour labels
      // 8 at a time (independent loads in flight), counted in list order
      uint32_t nx_slot = 0, nx_cat = 0;
      if (o0 + lane < o1) {
        nx_slot = a.pair_slot[o0 + lane - a.pair_base];
        nx_cat = a.pair_cat[o0 + lane - a.pair_base];
      }
      for (unsigned long long e0 = o0; e0 < o1; e0 += 32) {
        if (!__any_sync(FULL, unsat > 0)) break;
        const int ne = (int)min(32ull, o1 - e0);
        const uint32_t my_slot = nx_slot, my_cat = nx_cat;
        if (e0 + 32 + lane < o1) {
          nx_slot = a.pair_slot[e0 + 32 + lane - a.pair_base];
          nx_cat = a.pair_cat[e0 + 32 + lane - a.pair_base];
        }
        for (int j0 = 0; j0 < ne; j0 += 8) {
          uint32_t t8[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const uint32_t sl = __shfl_sync(FULL, my_slot, (j0 + u) & 31);
            t8[u] = (j0 + u < ne) ? lab[(uint64_t)sl << 5] : 0u;
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const uint32_t cat = __shfl_sync(FULL, my_cat, (j0 + u) & 31);
            if (j0 + u >= ne) break;
            if (DISJ) {
              const int q = ((const int8_t*)sTab)[row + t8[u]];
              if (q >= 0) {
                const int m = cnt[q * 32];
                if (m < kmax) {
                  const int kk = sK[m + 1];
                  if (kk >= 0) out[(q * nkI + kk) * 32] = (uint16_t)cat;
                  cnt[q * 32] = (uint8_t)(m + 1);
                  unsat -= (m + 1 == kmax);
                }
              }
            } else {
              uint32_t eb = ((const uint32_t*)sTab)[row + t8[u]];
              while (eb) {
                const int q = __ffs(eb) - 1;
                eb &= eb - 1;
                const int m = cnt[q * 32];
                if (m < kmax) {
                  const int kk = sK[m + 1];
                  if (kk >= 0) out[(q * nkI + kk) * 32] = (uint16_t)cat;
                  cnt[q * 32] = (uint8_t)(m + 1);
                  unsat -= (m + 1 == kmax);
                }
              }
            }
          }
        }
      }
      // the slots not met: misses of the sets, no slot beyond them
      for (int q = 0; q < a.nsmax; ++q) {
        const int got = cnt[q * 32];
        for (int kk = 0; kk < nkI; ++kk) {
          if (q < nset && got >= a.kvals[kk]) continue;
          out[(q * nkI + kk) * 32] = q < nset ? (uint16_t)a.cat_miss : (uint16_t)0xffff;
        }
      }
      a.rec_c[(uint64_t)li * 32 + lane] = c >= 0 ? (uint8_t)c : (uint8_t)0xff;
    }
  }
}

// Bin: one work item = (slot t = set q * nkI + order kk, range of centres).
// The block histograms that slot for all 32 realisations at once in shared
// memory laid out [nC][H][32], so lane r always hits bank r; the bins go to
// knn_core of realisation grp * 32 + r, set set_list[c][q], order kk.
__global__ void __launch_bounds__(1024, 1) k_knn_bin(KnnArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* hist = (uint32_t*)smem;                  // [cblk][H][32]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int NT = a.nsmax * a.nkI;
  // centre types are histogrammed a block of cblk types at a time when all
  // nC do not fit shared memory (records are then read once per block)
  const int cblk = a.cblk, ncb = (a.nC + cblk - 1) / cblk;
  const uint32_t nh = (uint32_t)cblk * a.H * 32;
  __shared__ uint32_t s_item;
  for (uint32_t i = threadIdx.x; i < nh; i += blockDim.x) hist[i] = 0;
  const uint32_t nranges = (a.cn + a.tile - 1) / a.tile;
  const uint32_t nitems = nranges * (uint32_t)NT * (uint32_t)ncb;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(a.work, 1u);
    __syncthreads();
    const uint32_t item = s_item;
    if (item >= nitems) break;
    const uint32_t range = item / (NT * ncb);
    const uint32_t rest = item - range * NT * ncb;
    const int t = (int)(rest / ncb);
    const int c_lo = (int)(rest - (uint32_t)t * ncb) * cblk;
    const uint32_t l0 = range * a.tile, l1 = min(l0 + a.tile, a.cn);
    // 8 centres per step: their loads are in flight together
    for (uint32_t lb = l0 + warp * 8; lb < l1; lb += nwarps * 8) {
      uint32_t v8[8], c8[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const uint32_t li = lb + u;
        v8[u] = 0xffff;
        c8[u] = 0xff;
        if (li < l1) {
          v8[u] = a.rec[((uint64_t)li * NT + t) * 32 + lane];
          c8[u] = a.rec_c[(uint64_t)li * 32 + lane];
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int cr = (int)c8[u] - c_lo;
        if (c8[u] != 0xff && v8[u] != 0xffff && cr >= 0 && cr < cblk)
          atomicAdd(&hist[((uint32_t)cr * a.H + v8[u]) * 32 + lane], 1u);
      }
    }
    __syncthreads();
    const int q = t / a.nkI, kk = t - q * a.nkI;
    for (uint32_t i = threadIdx.x; i < nh; i += blockDim.x) {
      const uint32_t v = hist[i];
      if (v) {
        hist[i] = 0;
        const int rr = a.grp * 32 + (int)(i & 31);
        const uint32_t cb = i >> 5;
        const int cr = (int)(cb / a.H), cat = (int)(cb - (uint32_t)cr * a.H);
        const int c = c_lo + cr;
        if (rr < a.nreal && c < a.nC && q < a.nsets[c]) {
          const int Sg = a.set_list[c * 32 + q];
          atomicAdd(&a.knn_core[((((uint64_t)rr * a.nC + c) * a.nS + Sg) * a.nkI + kk) * a.H + cat],
                    (unsigned long long)v);
        }
      }
    }
  }
}

// Realisation-major byte arrays src[rows][cols] to the group-major layout
// k_apply reads: dst[((r / G) * cols + c) * G + r % G], rows padded to a
// multiple of G with zeros.
__global__ void k_interleave(const uint8_t* __restrict__ src, uint64_t rows, uint64_t cols, int G,
                             uint8_t* __restrict__ dst) {
  const uint64_t rows_pad = (rows + G - 1) / G * G;
  const uint64_t total = cols * rows_pad;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t g = t / (cols * G), rem = t - g * cols * G;
    const uint64_t c = rem / G, r = g * G + (rem - c * G);
    dst[t] = r < rows ? src[r * cols + c] : 0;
  }
}

// centre_ok for ROI realisations: type is a target, and r_roi - |p - c| >= R
// evaluated in float as sqrt((px-cx)^2 + (py-cy)^2 + (pz-cz)^2).
__global__ void k_roi_mask(const float4* __restrict__ ions, const uint32_t* __restrict__ centres, uint32_t nc,
                           const float* __restrict__ rois, int nrois, float R, const uint8_t* __restrict__ labels,
                           const int8_t* __restrict__ cslot_of, uint8_t* __restrict__ ok) {
  const uint64_t total = (uint64_t)nc * nrois;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t q = (uint32_t)(t / nc), ci = (uint32_t)(t - (uint64_t)q * nc);
    const uint32_t s = centres[ci];
    const float4 p = ions[s];
    const float* c = rois + 4 * q;
    const float dd = sqrtf(dist2(p.x, p.y, p.z, c[0], c[1], c[2]));
    ok[t] = (cslot_of[labels[s]] >= 0) && (__fsub_rn(c[3], dd) >= R);
  }
}

__global__ void k_perm_mask(const uint8_t* __restrict__ lab, const uint32_t* __restrict__ centres, uint32_t nc,
                            const int8_t* __restrict__ cslot_of, uint8_t* __restrict__ ok) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nc; t += (uint64_t)gridDim.x * blockDim.x)
    ok[t] = cslot_of[lab[centres[t]]] >= 0;
}

void counted();

// FP64 audit: for each audited centre and each candidate within R (1 + 2^-10),
// the float distance the reference computes (sqrtf of the float d^2) is
// compared with the double-precision distance of the same coordinates, and
// the float bin (threshold table) with the bin of exact double arithmetic,
// floor((d64 - start) * nbins / (end - start)).  Out: [0] max |d32 - d64|,
// [1] max relative error (as double bits, atomicMax on ordered uint64), [2]
// pairs audited, [3] bin disagreements, [4] neighbour-set disagreements; up
// to cap disagreements are listed as (centre slot, neighbour slot, d32, d64).
struct AuditArgs {
  double start, scale, end, R64;
  int nbins;
  uint32_t stride;
  unsigned long long* out;
  uint32_t* list_slots;
  double* list_d;
  uint32_t cap;
};

__device__ __forceinline__ int cat64(double d, const AuditArgs& x) {
  if (d < x.start) return 0;
  if (d > x.end) return x.nbins + 1;
  const double b = floor((d - x.start) * x.scale);
  return b < (double)x.nbins ? 1 + (int)b : x.nbins + 1;
}

__global__ void __launch_bounds__(256) k_audit(ScanArgs a, AuditArgs x) {
  extern __shared__ __align__(16) unsigned char smem[];
  int8_t* rowtab = (int8_t*)smem;
  float* T = (float*)(smem + ((ROW_TABLE_ENTRIES * 2 + 15) & ~15));
  for (int i = threadIdx.x; i < ROW_TABLE_ENTRIES * 2; i += blockDim.x) rowtab[i] = a.rowtab[i];
  for (int i = threadIdx.x; i < a.H; i += blockDim.x) T[i] = a.cat_T[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const double R64 = x.R64;
  for (uint32_t ci = gw; ci < a.ncentres; ci += nw) {
    const uint32_t self = a.centres[(uint64_t)ci * x.stride];
    const float4 cp = a.ions[self];
    for_each_candidate(a, rowtab, cp, self, lane, [&](bool valid, uint32_t slot, float d2, bool inball, uint32_t,
                                                      bool) {
      if (!valid || slot == self) return;
      const float4 q = __ldg(a.ions + slot);
      const double dx = (double)cp.x - (double)q.x, dy = (double)cp.y - (double)q.y, dz = (double)cp.z - (double)q.z;
      const double d64 = sqrt(dx * dx + dy * dy + dz * dz);
      const bool in64 = d64 <= R64;
      if (!inball && !in64) return;
      if (inball != in64) {
        atomicAdd(&x.out[4], 1ull);
      } else {
        atomicAdd(&x.out[2], 1ull);
        const double d32 = (double)sqrtf(d2);
        const double err = fabs(d32 - d64);
        atomicMax(&x.out[0], (unsigned long long)__double_as_longlong(err));
        if (d64 > 0) atomicMax(&x.out[1], (unsigned long long)__double_as_longlong(err / d64));
        if (category(d2, T, a.H, a.guess_start, a.guess_scale) == cat64(d64, x)) return;
        atomicAdd(&x.out[3], 1ull);
      }
      const unsigned long long at = atomicAdd(&x.out[5], 1ull);
      if (at < x.cap) {
        x.list_slots[2 * at] = self;
        x.list_slots[2 * at + 1] = slot;
        x.list_d[2 * at] = (double)sqrtf(d2);
        x.list_d[2 * at + 1] = d64;
      }
    });
  }
}

void launch_audit(const ScanArgs& a, double start, double scale, double end, double R64, int nbins, uint32_t stride,
                  unsigned long long* out, uint32_t* list_slots, double* list_d, uint32_t cap, int sm_count,
                  cudaStream_t s) {
  AuditArgs x{start, scale, end, R64, nbins, stride, out, list_slots, list_d, cap};
  const size_t smem = ((ROW_TABLE_ENTRIES * 2 + 15) & ~15) + (size_t)a.H * 4;
  allow_dynamic_smem((const void*)k_audit, smem);
  counted();
  k_audit<<<sm_count * 4, 256, smem, s>>>(a, x);
}

// all ions j != self with d^2 <= R^2 in the full 3-D stencil (debug / parity)
__global__ void k_neighbors(const float4* __restrict__ ions, const uint32_t* __restrict__ cell_start, Grid g,
                            uint32_t self, float R, uint32_t* out_slot, float* out_d2, uint32_t cap,
                            uint32_t* count) {
  const float4 cp = ions[self];
  const float R2 = __fmul_rn(R, R);
  const float ext = R + g.margin;
  auto cl = [](int c, int n) { return c < 0 ? 0 : (c >= n ? n - 1 : c); };
  const int x0 = cl((int)floorf((cp.x - ext - g.lox) * g.inv_h), g.nx), x1 = cl((int)floorf((cp.x + ext - g.lox) * g.inv_h), g.nx);
  const int y0 = cl((int)floorf((cp.y - ext - g.loy) * g.inv_h), g.ny), y1 = cl((int)floorf((cp.y + ext - g.loy) * g.inv_h), g.ny);
  const int z0 = cl((int)floorf((cp.z - ext - g.loz) * g.inv_h), g.nz), z1 = cl((int)floorf((cp.z + ext - g.loz) * g.inv_h), g.nz);
  const int ny = y1 - y0 + 1, nz = z1 - z0 + 1;
  for (int r = blockIdx.x; r < ny * nz; r += gridDim.x) {
    const int yy = y0 + r % ny, zz = z0 + r / ny;
    const uint64_t cb = ((uint64_t)zz * g.ny + yy) * g.nx;
    const uint32_t s0 = cell_start[cb + x0], s1 = cell_start[cb + x1 + 1];
    for (uint32_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
      const float4 q = ions[s];
      const float d2 = dist2(cp.x, cp.y, cp.z, q.x, q.y, q.z);
      if (d2 <= R2 && s != self) {
        const uint32_t at = atomicAdd(count, 1u);
        if (at < cap) { out_slot[at] = s; out_d2[at] = d2; }
      }
    }
  }
}

// ------------------------------------------------------------------ launchers
// Every kernel this library launches is counted here (read via
// pp_kernel_launches), so a caller can verify that its work ran on the device.
static unsigned long long g_launches = 0;
void counted() { __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED); }
void scan_launched(int k) { __atomic_fetch_add(&g_launches, (unsigned long long)k, __ATOMIC_RELAXED); }
unsigned long long kernel_launches() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

inline unsigned grid_for(uint64_t n, int threads, unsigned cap = 152u * 16u) {
  uint64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned)(b > cap ? cap : b);
}

void launch_bbox(const float* xyz, uint64_t n, float* d_minmax, cudaStream_t s) {
  counted();
  k_bbox<<<grid_for(n, 256), 256, 0, s>>>(xyz, n, reinterpret_cast<uint32_t*>(d_minmax));
}

void launch_decode_pos(const uint32_t* be, uint64_t n, const float* lo, const float* hi, const uint8_t* type,
                       int nranges, float* xyz, uint8_t* label, cudaStream_t s) {
  counted();
  k_decode_pos<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const uint4*>(be), n, lo, hi, type, nranges, xyz, label);
}

void launch_cell_count(const float* xyz, uint64_t n, Grid g, uint32_t* cell_of, uint32_t* rank, uint32_t* counts,
                       cudaStream_t s) {
  counted();
  k_cell_count<<<grid_for(n, 256), 256, 0, s>>>(xyz, n, g, cell_of, rank, counts);
}

void launch_exclusive_scan_u32(uint32_t* data, uint64_t n, uint32_t* tmp, uint64_t tmp_elems, cudaStream_t s) {
  excl_scan<uint32_t>(data, n, tmp, tmp_elems, s);
}

void launch_exclusive_scan_u64_from_u32(const uint32_t* in, uint64_t n, unsigned long long* out,
                                        unsigned long long* tmp, uint64_t tmp_elems, cudaStream_t s) {
  counted();
  k_u32_to_u64<<<grid_for(n, 256), 256, 0, s>>>(in, n, out);
  excl_scan<unsigned long long>(out, n, tmp, tmp_elems, s);
}

void launch_scatter(const float* xyz, const uint8_t* label, uint64_t n, const uint32_t* cell_of, const uint32_t* rank,
                    const uint32_t* cell_start, float4* ions, uint32_t* slot_of_id, uint32_t* id_of_slot,
                    uint8_t* label_sorted, cudaStream_t s) {
  counted();
  k_scatter<<<grid_for(n, 256), 256, 0, s>>>(xyz, label, n, cell_of, rank, cell_start, ions, slot_of_id, id_of_slot);
  counted();
  k_labels_of_ions<<<grid_for(n, 256), 256, 0, s>>>(ions, n, label_sorted);
}

void launch_gather_labels(const uint8_t* src, const uint32_t* id_of_slot, uint64_t n, uint8_t* dst, int nsets,
                          cudaStream_t s) {
  counted();
  k_gather_labels<<<grid_for(n * (uint64_t)nsets, 256), 256, 0, s>>>(src, id_of_slot, n, dst, nsets);
}

void launch_permute_labels(const uint8_t* label_by_id, const uint32_t* perm, const uint32_t* id_of_slot, uint64_t n,
                           uint8_t* dst, cudaStream_t s) {
  counted();
  k_permute_labels<<<grid_for(n, 256), 256, 0, s>>>(label_by_id, perm, id_of_slot, n, dst);
}

void launch_surface_cells(const float4* ions, const uint32_t* cell_start, Grid g, int f, const float* tri_box,
                          const float* tri, const uint32_t* tcs, const uint32_t* tct, Grid tg, float rprime,
                          float* surf, cudaStream_t s) {
  counted();
  k_surface_cells<<<grid_for(tg.ncells * 32, kSurfWarps * 32), kSurfWarps * 32, 0, s>>>(ions, cell_start, g, f, tri_box,
                                                                                     tri, tcs, tct, tg, rprime, surf);
}

// number of cells holding at least one ion
__global__ void k_count_occupied(const uint32_t* __restrict__ cell_start, uint64_t ncells, unsigned long long* out) {
  unsigned long long c = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ncells; i += (uint64_t)gridDim.x * blockDim.x)
    c += cell_start[i + 1] > cell_start[i] ? 1ull : 0ull;
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(FULL, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

void launch_count_occupied(const uint32_t* cell_start, uint64_t ncells, unsigned long long* out, int sm_count,
                           cudaStream_t s) {
  counted();
  k_count_occupied<<<sm_count * 4, 256, 0, s>>>(cell_start, ncells, out);
}

void launch_nc_prefix(const uint32_t* cell_start, uint64_t ncells, const uint8_t* cflag, uint32_t* out,
                      uint32_t* scan_tmp, uint64_t scan_tmp_elems, cudaStream_t s) {
  counted();
  k_nc_count<<<grid_for(ncells + 1, 256), 256, 0, s>>>(cell_start, ncells, cflag, out);
  excl_scan<uint32_t>(out, ncells + 1, scan_tmp, scan_tmp_elems, s);
}

// Stencil rows (dy, dz), |dy|, |dz| <= s, per half-width s, sorted by
// dy^2 + dz^2 (ties by dz then dy) so a warp visits the nearest rows first.
const int8_t* row_table_host(int* entries) {
  struct Table {
    int8_t v[ROW_TABLE_ENTRIES * 2];
    Table() {
      for (int sr = 0; sr <= ROW_SMAX; ++sr) {
        int8_t* t = v + 2 * row_table_offset(sr);
        int k = 0;
        for (int d2 = 0; d2 <= 2 * sr * sr; ++d2)
          for (int dz = -sr; dz <= sr; ++dz)
            for (int dy = -sr; dy <= sr; ++dy)
              if (dy * dy + dz * dz == d2) { t[2 * k] = (int8_t)dy; t[2 * k + 1] = (int8_t)dz; ++k; }
      }
    }
  };
  static const Table table;  // built once, thread-safe initialisation
  if (entries) *entries = ROW_TABLE_ENTRIES;
  return table.v;
}

int launch_tri_bins(const float* tbox, uint64_t ntri, Grid tg, float grow, uint32_t* tstart, uint32_t* tfill,
                    uint32_t* tlist, uint64_t list_cap, uint32_t* scan_tmp, uint64_t scan_tmp_elems,
                    uint64_t* total_out, cudaStream_t s) {
  if (cudaMemsetAsync(tstart, 0, (tg.ncells + 1) * 4, s) != cudaSuccess) return -1;
  counted();
  k_tri_count<<<grid_for(ntri * 32, 256), 256, 0, s>>>(tbox, ntri, tg, grow, tstart);
  excl_scan<uint32_t>(tstart, tg.ncells + 1, scan_tmp, scan_tmp_elems, s);
  uint32_t total = 0;
  if (cudaMemcpyAsync(&total, tstart + tg.ncells, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  *total_out = total;
  if (total > list_cap) return 1;  // caller grows the list and calls again
  if (cudaMemcpyAsync(tfill, tstart, (tg.ncells + 1) * 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return -1;
  counted();
  k_tri_fill<<<grid_for(ntri * 32, 256), 256, 0, s>>>(tbox, ntri, tg, grow, tfill, tlist, list_cap, nullptr);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void launch_tri_entries(const float* tbox, uint64_t ntri, Grid tg, float grow, unsigned long long* total,
                        cudaStream_t s) {
  counted();
  k_tri_entries<<<grid_for(ntri, 256), 256, 0, s>>>(tbox, ntri, tg, grow, total);
}

void launch_voxel_count(const float* xyz, uint64_t n, const float* lo, float w, const uint32_t* nv, uint32_t* occ,
                        int* status, cudaStream_t s) {
  counted();
  k_voxel_count<<<grid_for(n, 256), 256, 0, s>>>(xyz, n, lo[0], lo[1], lo[2], w, nv[0], nv[1], nv[2], occ, status);
}

void launch_tri_box(const float* tri, uint64_t ntri, float* box, cudaStream_t s) {
  counted();
  k_tri_box<<<grid_for(ntri, 256), 256, 0, s>>>(tri, ntri, box);
}

void launch_surface_xyz(const float* xyz, uint64_t n, const float* tbox, const float* tri, const uint32_t* tstart,
                        const uint32_t* tlist, Grid tg, float rp, float* out, cudaStream_t s) {
  counted();
  k_surface_xyz<<<grid_for(n, 256), 256, 0, s>>>(xyz, n, tbox, tri, tstart, tlist, tg, rp, out);
}

void launch_select_centres(const uint8_t* labels, const float* surf, uint64_t n, float R2, const int8_t* cslot_of,
                           const uint8_t* extra, uint32_t* flags, uint32_t* scan_tmp, uint64_t scan_tmp_elems,
                           uint32_t* out, uint32_t* count, uint8_t* cflag, cudaStream_t s) {
  counted();
  k_select_flags<<<grid_for(n + 1, 256), 256, 0, s>>>(labels, surf, n, R2, cslot_of, extra, flags, cflag);
  excl_scan<uint32_t>(flags, n + 1, scan_tmp, scan_tmp_elems, s);
  counted();
  k_select_write<<<grid_for(n, 256), 256, 0, s>>>(labels, surf, n, R2, cslot_of, extra, flags, out, count);
}

template <int KR, int EMAX>
static int launch_scan_t(const ScanArgs& a, int sm_count, size_t smem, cudaStream_t s) {
  auto kern = k_scan<KR, EMAX>;
  if (smem > 48 * 1024) {
    if (!allow_dynamic_smem((const void*)kern, smem)) return -1;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess || per_sm < 1) return -1;
  const int blocks = sm_count * per_sm;
  counted();
  kern<<<blocks, 256, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_scan(const ScanArgs& a, int kr, int emax, int sm_count, size_t* smem_used, cudaStream_t s) {
  const int nwarps = 8;
  size_t smem = 16 + ROW_TABLE_ENTRIES * 2 + (size_t)((a.H + 4) & ~3) * 4 + (size_t)((a.lut_n + 7) & ~7) * 2 + 512;
  if (kr > 0) smem += (size_t)a.nC * 256 * 4;
  if (kr > 0 && a.disjoint) smem += (size_t)nwarps * a.emax * (kr * 32 + 1) * 4;
  if (a.rdf_in_smem) smem += (size_t)a.nC * a.nE * a.H * 4;
  if (a.flags & PP_CNTNB) smem += (size_t)nwarps * a.nE * 4;
  if (a.mode == 2) smem += (size_t)nwarps * a.H * 4;
  if (kr > 0 && a.disjoint) smem += (size_t)a.nC * 256;
  if (smem_used) *smem_used = smem;
  if (kr == 0) return launch_scan_t<0, 1>(a, sm_count, smem, s);
  if (a.disjoint) {
    if (kr == 1) return launch_scan_t<1, 0>(a, sm_count, smem, s);
    if (kr <= 4) return launch_scan_t<4, 0>(a, sm_count, smem, s);
  }
  if (kr == 1) {
    if (emax <= 1) return launch_scan_t<1, 1>(a, sm_count, smem, s);
    if (emax <= 8) return launch_scan_t<1, 8>(a, sm_count, smem, s);
    return launch_scan_t<1, 32>(a, sm_count, smem, s);
  }
  if (kr <= 4) {
    if (emax <= 1) return launch_scan_t<4, 1>(a, sm_count, smem, s);
    if (emax <= 8) return launch_scan_t<4, 8>(a, sm_count, smem, s);
  }
  return -2;
}

void launch_cmask_or(const float* surf, uint64_t n, const float* R2, const uint32_t* bits, int nb, uint32_t* cmask,
                     cudaStream_t s) {
  counted();
  k_cmask_or<<<grid_for(n, 256), 256, 0, s>>>(surf, n, R2, bits, nb, cmask);
}

void launch_multi_select(const uint8_t* labels, const uint32_t* cmask, const uint32_t* q_of_type, uint64_t n,
                         uint32_t* flags, uint32_t* scan_tmp, uint64_t scan_tmp_elems, uint32_t* out, uint32_t* count,
                         cudaStream_t s) {
  counted();
  k_multi_flags<<<grid_for(n + 1, 256), 256, 0, s>>>(labels, cmask, q_of_type, n, flags);
  excl_scan<uint32_t>(flags, n + 1, scan_tmp, scan_tmp_elems, s);
  counted();
  k_multi_write<<<grid_for(n, 256), 256, 0, s>>>(labels, cmask, q_of_type, n, flags, out, count);
}

static size_t multi_smem(const MultiArgs& m, uint32_t rdf_words) {
  return 16 + kMultiMaxQueries * 2 * 8 + ((sizeof(MultiQuery) * kMultiMaxQueries + 15) & ~size_t(15)) +
         ((sizeof(MultiTask) * kMultiMaxTasks + 15) & ~size_t(15)) + 256 * 8 * 2 + kMultiMaxQueries * 8 + 256 * 4 +
         (size_t)kMultiWarps * kMultiMaxQueries * 4 + ((ROW_TABLE_ENTRIES * 2 + 15) & ~15) +
         (size_t)kMultiWarps * m.lists * 32 * 4 + (size_t)rdf_words * 4;
}

int launch_multi(const MultiArgs& m0, int sm_count, size_t* smem_used, cudaStream_t s) {
  if (m0.nq < 1 || m0.nq > kMultiMaxQueries || m0.nt < 1 || m0.nt > kMultiMaxTasks || m0.lists < 0 ||
      m0.lists > kMultiMaxTasks)
    return -3;
  MultiArgs m = m0;
  // RDF counters in shared memory when they fit beside the lists, else
  // straight to the global cores
  size_t smem = multi_smem(m, m.rdf_words);
  if (smem > 160 * 1024) {
    m.rdf_words = 0;
    smem = multi_smem(m, 0);
  }
  if (smem_used) *smem_used = smem;
  if (smem > 220 * 1024) return -3;
  if (!allow_dynamic_smem((const void*)k_multi, smem)) return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_multi, kMultiWarps * 32, smem) != cudaSuccess ||
      per_sm < 1)
    return -1;
  counted();
  k_multi<<<sm_count * per_sm, kMultiWarps * 32, smem, s>>>(m);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void launch_ball_count(const ScanArgs& a, const uint32_t* id_of_slot, uint64_t n, uint32_t* count_by_id, int sm_count,
                       cudaStream_t s) {
  counted();
  k_ball_count<<<sm_count * 8, 256, 0, s>>>(a, id_of_slot, n, count_by_id);
}

void launch_guard(const ScanArgs& a, const uint8_t* clus, uint8_t* guard_then_labels, uint64_t n, int sm_count,
                  cudaStream_t s) {
  counted();
  k_guard<<<sm_count * 8, 256, 0, s>>>(a, clus, guard_then_labels, n);
  counted();
  k_cluster_labels<<<grid_for(n, 256), 256, 0, s>>>(clus, n, guard_then_labels);
}

int launch_npcorr(const ScanArgs& a, const NpcArgs& p, int sm_count, cudaStream_t s) {
  const int nwarps = 8;
  const size_t smem = (size_t)nwarps * a.emax * 32 * 12 + (size_t)a.nC * 256 * 4 + ROW_TABLE_ENTRIES * 2 + 256;
  if (p.K < 1 || p.K > 32 || smem > 200 * 1024) return -2;
  if (smem > 48 * 1024 &&
      !allow_dynamic_smem((const void*)k_npcorr, smem))
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_npcorr, nwarps * 32, smem) != cudaSuccess || per_sm < 1)
    return -1;
  counted();
  k_npcorr<<<sm_count * per_sm, nwarps * 32, smem, s>>>(a, p);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t brick_smem(const ScanArgs& a, bool knn) {
  constexpr int NW = 8;
  size_t b = 16 + NW * 32 * 16 + NW * 32 * 4 + (size_t)((a.H + 3) & ~3) * 4 + (size_t)((a.lut_n + 7) & ~7) * 2;
  if (a.rdf_in_smem) b += (size_t)a.nC * a.nE * a.H * 4;
  if (knn) b += (size_t)NW * a.emax * a.bcap * a.kmax * 4;
  b += ROW_TABLE_ENTRIES * 2 + 512 + 2 * NW * 32;
  if (knn) b += (size_t)a.nC * 256;
  return b;
}

int launch_brick(const ScanArgs& a, int kr, int sm_count, size_t* smem_used, cudaStream_t s) {
  const bool knn = kr > 0;
  if (a.mode != 0 || (a.flags & PP_CNTNB) || kr > 1 || (knn && !a.disjoint) || a.bx < 1 || a.bcap < 1 || a.bcap > 32)
    return -3;
  const size_t smem = brick_smem(a, knn);
  if (smem_used) *smem_used = smem;
  if (smem > 200 * 1024) return -3;
  auto kern = knn ? k_brick<true> : k_brick<false>;
  if (!allow_dynamic_smem((const void*)kern, smem))
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess || per_sm < 1) return -1;
  counted();
  kern<<<sm_count * per_sm, 256, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t lanes_smem(const ScanArgs& a) {
  constexpr int NW = kLanesWarps;
  size_t b = 16 + 2 * NW * 32 * 16 + NW * 2 * 16 + 2 * NW * 32 * 4 + NW * 1024 * 2 + (size_t)((a.H + 4) & ~3) * 4;
  if (a.rdf_in_smem) b += (size_t)a.nC * a.nE * a.H * 4;
  b += (size_t)((a.lut_n + 7) & ~7) * 2 + 512;
  return b;
}

int launch_lanes(const ScanArgs& a, int kr, int sm_count, size_t* smem_used, cudaStream_t s) {
  if (a.mode != 0 || kr > 0 || (a.flags & PP_CNTNB) || !(a.flags & PP_RDF) || a.bx < 1 || a.by < 1 || a.bz < 1 ||
      a.nC > 254 || a.nE > 254 || !a.brows)
    return -3;
  const size_t smem = lanes_smem(a);
  if (smem_used) *smem_used = smem;
  if (smem > 200 * 1024) return -3;
  auto kern = a.sym ? (a.rdf_in_smem ? k_lanes<true, true> : k_lanes<true, false>)
                    : (a.rdf_in_smem ? k_lanes<false, true> : k_lanes<false, false>);
  if (!allow_dynamic_smem((const void*)kern, smem))
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kLanesWarps * 32, smem) != cudaSuccess ||
      per_sm < 1)
    return -1;
  counted();
  kern<<<sm_count * per_sm, kLanesWarps * 32, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t lanes_knn_smem(const ScanArgs& a, bool cat) {
  constexpr int NW = kLanesKnnWarps;
  const size_t em = a.emax > 1 ? a.emax : 1;
  const size_t frows = cat ? em + 1 : em * a.kmax + 1;
  const size_t crows = cat ? (((size_t)NW * em * a.kmax * 32 * 2 + 15) & ~size_t(15)) : 0;
  return NW * 32 * 16 + NW * 2 * 16 + NW * 32 * 4 + (size_t)NW * frows * 32 * 4 + crows + (size_t)((a.H + 4) & ~3) * 4 +
         (size_t)((a.lut_n + 7) & ~7) * 2 + 256 + 256 * 4;
}

int launch_lanes_knn(const ScanArgs& a, bool disjoint_sets, int sm_count, size_t* smem_used, cudaStream_t s) {
  if (a.mode != 0 || (a.flags & (PP_CNTNB | PP_RDF)) || !disjoint_sets || a.kmax < 1 || a.kmax > 64 || a.bx < 1 ||
      a.by < 1 || a.bz < 1 || !a.brows || a.nC > 8 || a.emax > 15)  // sets packed 4 bits per centre slot
    return -3;
  // d^2 lists while they leave room for two blocks of 8 warps per SM;
  // category lists beyond that (e.g. 8 sets of k = 20: 20.6 KB a warp as d^2,
  // 11.4 KB as categories); one block per SM for the largest
  bool cat = a.lists_mode == 2;
  size_t smem = lanes_knn_smem(a, cat);
  if (!cat && a.lists_mode == 0 && smem > 110 * 1024 && lanes_knn_smem(a, true) < smem) {
    cat = true;
    smem = lanes_knn_smem(a, true);
  }
  if (smem_used) *smem_used = smem;
  if (smem > 200 * 1024 || (cat && a.H > 65535)) return -3;
  const bool uni = a.uniform_sets != 0;
#define PP_KNN_KERN(KBV) \
  (cat ? (uni ? k_lanes_knn<KBV, true, true> : k_lanes_knn<KBV, false, true>) \
       : (uni ? k_lanes_knn<KBV, true, false> : k_lanes_knn<KBV, false, false>))
  auto kern = a.kmax <= 8    ? PP_KNN_KERN(8)
              : a.kmax <= 10 ? PP_KNN_KERN(10)
              : a.kmax <= 16 ? PP_KNN_KERN(16)
              : a.kmax <= 20 ? PP_KNN_KERN(20)
                             : PP_KNN_KERN(0);
#undef PP_KNN_KERN
  if (!allow_dynamic_smem((const void*)kern, smem))
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kLanesKnnWarps * 32, smem) != cudaSuccess ||
      per_sm < 1)
    return -1;
  counted();
  kern<<<sm_count * per_sm, kLanesKnnWarps * 32, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int G, bool KS>
static int launch_apply_t(const ApplyArgs& a, int sm_count, size_t smem, cudaStream_t s) {
  auto kern = k_apply<G, KS>;
  if (smem > 48 * 1024) {
    if (!allow_dynamic_smem((const void*)kern, smem)) return -1;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kApplyThreads, smem) != cudaSuccess || per_sm < 1)
    return -1;
  counted();
  kern<<<sm_count * per_sm, kApplyThreads, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

static size_t apply_bytes(const ApplyArgs& a, int G, bool ks) {
  return ApplyLayout(a, G, ks).bytes(G, kApplyThreads / 32, std::max(a.nsmax, 1));
}

int apply_configure(ApplyArgs& a) {
  const size_t cap = 220 * 1024;
  const bool knn = (a.flags & PP_MKNN) != 0;
  for (int pass = knn ? 0 : 1; pass < 2; ++pass) {
    const bool ks = pass == 0;
    for (int G = 8; G >= 1; G >>= 1) {
      if (apply_bytes(a, G, ks) <= cap) {
        a.group = G;
        a.knn_smem = ks ? 1 : 0;
        return 0;
      }
    }
  }
  return -2;
}

int launch_apply(const ApplyArgs& a, int sm_count, cudaStream_t s) {
  const int G = a.group;
  const bool ks = a.knn_smem != 0;
  const size_t smem = apply_bytes(a, G, ks);
  if (ks) {
    if (G == 8) return launch_apply_t<8, true>(a, sm_count, smem, s);
    if (G == 4) return launch_apply_t<4, true>(a, sm_count, smem, s);
    if (G == 2) return launch_apply_t<2, true>(a, sm_count, smem, s);
    return launch_apply_t<1, true>(a, sm_count, smem, s);
  }
  if (G == 8) return launch_apply_t<8, false>(a, sm_count, smem, s);
  if (G == 4) return launch_apply_t<4, false>(a, sm_count, smem, s);
  if (G == 2) return launch_apply_t<2, false>(a, sm_count, smem, s);
  return launch_apply_t<1, false>(a, sm_count, smem, s);
}

__global__ void k_max_u32(const uint32_t* __restrict__ v, uint64_t n, uint32_t* out) {
  uint32_t m = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, v[i]);
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(FULL, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

void launch_max_u32(const uint32_t* v, uint64_t n, uint32_t* out, cudaStream_t s) {
  counted();
  k_max_u32<<<grid_for(n, 256), 256, 0, s>>>(v, n, out);
}

static size_t knn_walk_bytes(const KnnArgs& k, int nwarps) {
  return (size_t)(k.nC + 1) * 256 * (k.disjoint ? 1 : 4) + (size_t)k.nC * 4 + 512 +
         (size_t)nwarps * k.nsmax * 32;
}

static int knn_walk_warps(const KnnArgs& k) {
  for (int w = 16; w >= 2; w /= 2)
    if (knn_walk_bytes(k, w) <= 96 * 1024) return w;
  return 0;
}

int knn32_check(KnnArgs& k) {
  if (k.nsmax > 32 || k.kmax > 254 || k.nC > 254) return -2;
  if (!knn_walk_warps(k)) return -2;
  // centre types per bin histogram block
  const size_t per_type = (size_t)k.H * 32 * 4;
  if (per_type > 200 * 1024) return -2;
  k.cblk = (int)std::min<size_t>((size_t)k.nC, (200 * 1024) / per_type);
  return 0;
}

int launch_knn_walk(const KnnArgs& k, int sm_count, cudaStream_t s) {
  const int w = knn_walk_warps(k);
  if (!w) return -2;
  const size_t smem = knn_walk_bytes(k, w);
  auto kern = k.disjoint ? k_knn_walk<true> : k_knn_walk<false>;
  if (!allow_dynamic_smem((const void*)kern, smem))
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, w * 32, smem) != cudaSuccess || per_sm < 1)
    return -1;
  counted();
  kern<<<sm_count * per_sm, w * 32, smem, s>>>(k);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_knn_bin(const KnnArgs& k, int sm_count, cudaStream_t s) {
  if (k.cblk < 1) return -2;
  const size_t smem = (size_t)k.cblk * k.H * 32 * 4;
  if (smem > 200 * 1024) return -2;
  if (smem > 48 * 1024 &&
      !allow_dynamic_smem((const void*)k_knn_bin, smem))
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_knn_bin, 1024, smem) != cudaSuccess || per_sm < 1)
    return -1;
  counted();
  k_knn_bin<<<sm_count * per_sm, 1024, smem, s>>>(k);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void launch_interleave(const uint8_t* src, uint64_t rows, uint64_t cols, int G, uint8_t* dst, cudaStream_t s) {
  counted();
  k_interleave<<<grid_for(cols * ((rows + G - 1) / G * G), 256), 256, 0, s>>>(src, rows, cols, G, dst);
}

void launch_roi_mask(const float4* ions, const uint32_t* centres, uint32_t nc, const float* rois, int nrois, float R,
                     const uint8_t* labels, const int8_t* cslot_of, uint8_t* ok, cudaStream_t s) {
  counted();
  k_roi_mask<<<grid_for((uint64_t)nc * nrois, 256), 256, 0, s>>>(ions, centres, nc, rois, nrois, R, labels, cslot_of, ok);
}

void launch_perm_mask(const uint8_t* lab, const uint32_t* centres, uint32_t nc, const int8_t* cslot_of, uint8_t* ok,
                      cudaStream_t s) {
  counted();
  k_perm_mask<<<grid_for(nc, 256), 256, 0, s>>>(lab, centres, nc, cslot_of, ok);
}

void launch_neighbors(const float4* ions, const uint32_t* cell_start, Grid g, uint32_t self, float R,
                      const uint32_t* id_of_slot, uint32_t* out_slot, float* out_d2, uint32_t cap, uint32_t* count,
                      cudaStream_t s) {
  (void)id_of_slot;
  counted();
  k_neighbors<<<64, 256, 0, s>>>(ions, cell_start, g, self, R, out_slot, out_d2, cap, count);
}

}  // namespace pp

// ------------------------------------------------------------- small helpers
namespace pp_host {

__global__ void k_gather_f32(const float* __restrict__ src, const uint32_t* __restrict__ id_of_slot, uint64_t n,
                             float* __restrict__ dst) {
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x)
    dst[s] = src[id_of_slot[s]];
}

__global__ void k_fill_f32(float* __restrict__ dst, uint64_t n, float v) {
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x)
    dst[s] = v;
}

void gather_f32_sorted(const float* src, const uint32_t* id_of_slot, uint64_t n, float* dst, cudaStream_t s) {
  pp::counted();
  k_gather_f32<<<pp::grid_for(n, 256), 256, 0, s>>>(src, id_of_slot, n, dst);
}

void fill_f32(float* dst, uint64_t n, float v, cudaStream_t s) {
  pp::counted();
  k_fill_f32<<<pp::grid_for(n, 256), 256, 0, s>>>(dst, n, v);
}

}  // namespace pp_host
