// Hull distance (ion2surf) for callers that cannot allocate device memory:
// pp_surfdist_noalloc.
//
// Who needs it: a host program that hands the whole device to its own memory
// pool at start-up (a cudaMalloc of ours would fail, or fragment the pool
// behind the owner's back), and a latency-bound loop that may not pay the
// device-wide synchronisation cudaFree implies.  Such a caller passes its own
// device buffers for the inputs and the output; every other buffer the pass
// needs -- the triangle boxes, the triangle grid, its per-cell lists and the
// prefix-scan partials -- lives in one file-scope __device__ array of fixed
// size.  Each GPU on which this file's module is loaded holds that array
// (64 MiB) until the process exits.  The CUDA runtime loads modules lazily by
// default (CUDA_MODULE_LOADING=LAZY), and this module holds no kernel, so the
// array is given device memory at the first call on a device, when the call
// looks its address up.  A caller whose pool takes the whole device makes one
// call with n = 0 on each device before that (it only does the set-up).  The
// address is cached per device for the life of the process: after
// cudaDeviceReset, or once the primary context is destroyed and created
// again, the cached address is stale and this entry point must not be used.
//
// The entry point calls no cudaMalloc, cudaFree or allocating library routine
// and allocates no host memory either.  It uses cudaMemsetAsync, plain
// cudaMemcpyAsync of a few bytes to the caller's stack and stream
// synchronisation, which allocate nothing.
//
// The array is shared by every call on a device and keeps what the last call
// left there; each call clears what must start at zero (the box reduction,
// the list-entry total, the per-cell counts).  Calls whose GPU work overlaps
// -- issued on different streams, or from several threads without ordering --
// race on the array: issue them on one stream or synchronise between them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "paraprobe_gb300.h"
#include "pp_host.h"
#include "pp_internal.h"

// Size of the shared scratch, and the largest hull it is sized for.
#define PP_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define PP_NOALLOC_MAX_TRIANGLES 2000000ull

static __device__ __align__(256) unsigned char g_noalloc_scratch[PP_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;                        // guards g_base and serialises the host side of calls
unsigned char* g_base[kMaxDevices];     // device address of g_noalloc_scratch, per device

int say(char* err, size_t cap, int code, const char* fmt, ...) {
  if (err && cap) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(err, cap, fmt, ap);
    va_end(ap);
  }
  return code;
}

// Set-up, once per device, with that device current: the array's device
// address.  (In host code the array's name only stands in for the symbol.)
int scratch_base(int dev, unsigned char** out, char* err, size_t cap) {
  if (dev < 0 || dev >= kMaxDevices)
    return say(err, cap, PP_ERR_UNSUPPORTED, "device %d is beyond the %d devices this entry point tracks", dev,
               kMaxDevices);
  if (!g_base[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return say(err, cap, PP_ERR_CUDA, "cudaGetSymbolAddress of the scratch failed: %s", cudaGetErrorString(e));
    g_base[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_base[dev];
  return PP_OK;
}

bool device_memory(const void* p, int dev) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}

float key_to_float(uint32_t o) {
  const uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

constexpr size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// Scratch layout: [0, 256) box reduction (32 B) and list-entry total (at 64);
// then triangle boxes, cell starts, fill cursors, scan partials, cell lists.
struct Layout {
  size_t box = 256, start = 0, fill = 0, scan = 0, list = 0;
  uint64_t scan_elems = 0, list_cap = 0;
  bool fits = false;
  Layout(uint64_t ntri, uint64_t ncells) {
    start = up256(box + 24 * ntri);
    fill = up256(start + 4 * (ncells + 1));
    scan_elems = 2 * ((ncells + 1) / 2048 + 64);
    scan = up256(fill + 4 * (ncells + 1));
    list = up256(scan + 4 * scan_elems);
    fits = list + 4 * ntri <= PP_NOALLOC_SCRATCH_BYTES;
    list_cap = fits ? (PP_NOALLOC_SCRATCH_BYTES - list) / 4 : 0;
  }
};

}  // namespace

extern "C" int pp_surfdist_noalloc(const float* xyz, uint64_t n, const float* tri, uint64_t ntri, float rp,
                                   float* d2_out, void* stream, char* err, size_t err_cap) {
  if (err && err_cap) err[0] = '\0';
  if (!(rp > 0.f) || !std::isfinite(rp)) return say(err, err_cap, PP_ERR_INVALID, "R' must be finite and positive");
  if (n && (!xyz || !d2_out)) return say(err, err_cap, PP_ERR_INVALID, "xyz and d2_out are required");
  if (ntri && !tri) return say(err, err_cap, PP_ERR_INVALID, "tri is required when ntri > 0");
  if (ntri > PP_NOALLOC_MAX_TRIANGLES)
    return say(err, err_cap, PP_ERR_UNSUPPORTED,
               "%llu triangles exceed the %llu that the %llu MiB static scratch of pp_surfdist_noalloc takes",
               (unsigned long long)ntri, PP_NOALLOC_MAX_TRIANGLES, PP_NOALLOC_SCRATCH_BYTES >> 20);
  std::lock_guard<std::mutex> lock(g_mu);
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return say(err, err_cap, PP_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(e));
  unsigned char* base = nullptr;
  int rc = scratch_base(dev, &base, err, err_cap);
  if (rc) return rc;
  if (n == 0) return PP_OK;
  if (!device_memory(xyz, dev) || !device_memory(d2_out, dev) || (ntri && !device_memory(tri, dev)))
    return say(err, err_cap, PP_ERR_INVALID, "xyz, tri and d2_out must be device memory of the current device (%d)",
               dev);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
#define NA_CK(call)                                                                                        \
  do {                                                                                                     \
    const cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return say(err, err_cap, PP_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)
  if (ntri == 0) {  // no hull: every ion is R' away from it
    pp_host::fill_f32(d2_out, n, rp * rp, s);
    NA_CK(cudaGetLastError());
    return PP_OK;
  }
  // vertex box (order-preserving keys: min x,y,z, max x,y,z, non-finite count)
  uint32_t* keys = reinterpret_cast<uint32_t*>(base);
  NA_CK(cudaMemsetAsync(keys, 0xff, 12, s));
  NA_CK(cudaMemsetAsync(keys + 3, 0, 20, s));
  pp::launch_bbox(tri, 3 * ntri, reinterpret_cast<float*>(keys), s);
  float* box = reinterpret_cast<float*>(base + 256);
  pp::launch_tri_box(tri, ntri, box, s);
  uint32_t bb[8];
  NA_CK(cudaMemcpyAsync(bb, keys, sizeof bb, cudaMemcpyDeviceToHost, s));
  NA_CK(cudaStreamSynchronize(s));
  if (bb[6]) return say(err, err_cap, PP_ERR_INVALID, "the hull has %u non-finite coordinates", bb[6]);
  float glo[3], ghi[3];
  for (int k = 0; k < 3; ++k) { glo[k] = key_to_float(bb[k]); ghi[k] = key_to_float(bb[3 + k]); }
  // grid geometry as for a hull uploaded with pp_hull_upload: boxes grown by
  // R' + slack; coarser cells until the lists fit the scratch
  float mag = 0.f;
  for (int k = 0; k < 3; ++k) mag = std::fmax(mag, std::fmax(std::fabs(glo[k]), std::fabs(ghi[k])));
  const float slack = 1e-3f + 1e-5f * mag;
  const float grow = rp + slack;
  for (int k = 0; k < 3; ++k) { glo[k] -= grow + slack; ghi[k] += grow + slack; }
  unsigned long long* total_dev = reinterpret_cast<unsigned long long*>(base + 64);
  // The cell edge is searched for scratch fit, not by the allocating path's
  // cell-count rule, so the two grids may differ.  The result does not depend
  // on the grid: every triangle whose box grown by R' + slack reaches a cell
  // is listed there, so each ion meets every triangle within R' of it and
  // takes the same minimum over the same float distances.
  double h = std::fmax((double)rp, 0.25);
  pp::Grid tg{};
  Layout L(ntri, 0);
  bool placed = false;
  for (int attempt = 0; attempt < 96 && !placed; ++attempt, h *= 1.25) {
    double cells = 1;
    int nd[3];
    for (int k = 0; k < 3; ++k) {
      const double c = std::floor((ghi[k] - glo[k]) / h) + 1;
      cells *= c;
      nd[k] = c < 2.0e9 ? (int)c : 0;
    }
    if (!nd[0] || !nd[1] || !nd[2] || cells > 2.0e9) continue;
    L = Layout(ntri, (uint64_t)cells);
    if (!L.fits) continue;
    tg = pp::Grid{};
    tg.h = (float)h;
    tg.inv_h = (float)(1.0 / h);
    tg.lox = glo[0]; tg.loy = glo[1]; tg.loz = glo[2];
    tg.nx = nd[0]; tg.ny = nd[1]; tg.nz = nd[2];
    tg.ncells = (uint64_t)cells;
    unsigned long long entries = 0;
    NA_CK(cudaMemsetAsync(total_dev, 0, 8, s));
    pp::launch_tri_entries(box, ntri, tg, grow, total_dev, s);
    NA_CK(cudaMemcpyAsync(&entries, total_dev, 8, cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    if (entries > L.list_cap) continue;
    placed = true;
  }
  if (!placed)
    return say(err, err_cap, PP_ERR_OVERFLOW, "the triangle lists of this hull do not fit the %llu MiB static scratch",
               PP_NOALLOC_SCRATCH_BYTES >> 20);
  uint32_t* start = reinterpret_cast<uint32_t*>(base + L.start);
  uint32_t* fill = reinterpret_cast<uint32_t*>(base + L.fill);
  uint32_t* scan = reinterpret_cast<uint32_t*>(base + L.scan);
  uint32_t* list = reinterpret_cast<uint32_t*>(base + L.list);
  uint64_t got = 0;
  rc = pp::launch_tri_bins(box, ntri, tg, grow, start, fill, list, L.list_cap, scan, L.scan_elems, &got, s);
  if (rc) return say(err, err_cap, PP_ERR_CUDA, "triangle binning failed (%d)", rc);
  pp::launch_surface_xyz(xyz, n, box, tri, start, list, tg, rp, d2_out, s);
  NA_CK(cudaGetLastError());
#undef NA_CK
  return PP_OK;
}
