// pp_capi.cu -- host side of the C ABI in include/paraprobe_gb300.h.
//
// A context owns every device buffer.  A cloud keeps its input-order copy
// (xyz, labels) plus the cell-sorted layout the kernels read; the cell grid is
// (re)built lazily when a query's radius needs a different cell edge.  Each
// run prepares small host tables (bin thresholds, type slots, environment
// sets), launches the kernels on the caller's stream, and the fetch calls fold
// the per-type "core" histograms into the per-task histograms of
// compute_generic_spatstat3 (src/PARAPROBE_SolverHdl.cpp:3685-4177).

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/paraprobe_gb300.h"
#include "pp_internal.h"
#include "pp_host.h"

using pp::Grid;

namespace {

constexpr double kEpsilon = 1.0e-6;  // src/PARAPROBE_Numerics.h:44
constexpr size_t kSpareClouds = 2;    // freed clouds whose device buffers a context keeps

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    release();
    if (b == 0) b = 16;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    else p = nullptr;
    return e;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Page-locked host staging (result downloads), grown on demand.
struct PinBuf {
  void* p = nullptr;
  size_t bytes = 0;
  PinBuf() = default;
  PinBuf(const PinBuf&) = delete;
  PinBuf& operator=(const PinBuf&) = delete;
  ~PinBuf() { release(); }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMallocHost(&p, b);
    if (e == cudaSuccess) bytes = b;
    else p = nullptr;
    return e;
  }
};

struct Hull {
  std::vector<float> tri;  // ntri * 9
  float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};  // bounds of the vertices
  float carve = 2.0f;
  bool present = false;
};

struct Cloud {
  uint64_t n = 0;
  DevBuf xyz, label;            // input order
  std::vector<uint32_t> ids;    // caller ids (empty = input index)
  // grid
  bool grid_ok = false;
  Grid g{};
  uint64_t grid_version = 0;
  DevBuf ions, cell_start, slot_of_id, id_of_slot, label_sorted;
  // hull / ion2surf
  // tuning (pp_autotune): cell edge = R / cell_ratio, centres per block tile
  float cell_ratio = 4.0f;
  uint32_t tile = 128;
  // brick scan: (cells per brick << 16) | centres per warp batch; 0 = the
  // per-centre scan with `tile` centres per block work item
  uint32_t brick = 0;
  // RDF / RIPK passes: cell block (x, y, z) of the centre-per-lane scan
  // (0 = the defaults below)
  uint32_t lanes_bx = 0, lanes_by = 0, lanes_bz = 0;
  uint64_t occupied = 0;  // non-empty cells of the grid
  // the cell block was set by pp_cloud_prepare rather than by tuning: passes
  // take it only where centres are dense enough to fill a warp (default_block)
  bool lanes_auto = false;
  std::vector<uint64_t> type_count;  // ions of each type (pp_cloud_prepare)
  Hull hull;
  DevBuf user_surf;             // input order, when given
  bool has_user_surf = false;
  DevBuf surf;                  // sorted order, valid for (surf_rp, surf_version)
  float surf_rp = -1.f;
  uint64_t surf_version = ~0ull;
  DevBuf tri_dev, tri_box, tcell_start, tcell_list;
  Grid tg{};                    // hull grid: the ion grid coarsened tri_f times per axis
  int tri_f = 1;
  uint64_t tri_grid_version = ~0ull;
  float tri_grow = -1.f, tri_slack = 0.f;
  bool tri_ok = false;
};

struct Tables {
  // histogram
  float rmin = 0.f, rincr = 0.1f, rmax = 2.f;  // reference defaults, src/PARAPROBE_Settings.cpp:106-108
  uint32_t nbins = 0;
  double hstart = 0, hend = 0, hscale = 0;
};

struct RunPlan {
  uint32_t flags = 0;
  int H = 0;
  std::vector<uint32_t> kvals;     // internal sorted unique ks
  std::vector<uint32_t> k_out;     // MKNN k list as given
  int nC = 0, nE = 0, nS = 0;
  std::vector<int> ctype, etype;   // slot -> type
  std::vector<int8_t> cslot_of, eslot_of;
  std::vector<std::vector<uint32_t>> sets;  // global env sets as type lists (mask words)
  std::vector<int> task_set;       // task -> global set id
  std::vector<uint32_t> envbits;   // [nC][256]
  std::vector<int> set_list;       // [nC][32]
  std::vector<int> nsets;          // [nC]
  int emax = 0, kr = 0, kmax = 0;
  int cmax = 0;
  int cat_miss = 0;
  std::vector<float> catT;
  std::vector<uint16_t> lut;       // category by high bits of d^2 (see build_lut)
  // n-point correlations: tasks per centre type with their local env set
  std::vector<int> ntk, tk_task, tk_set;  // [nC], [nC][32], [nC][32]
  int npc_half = 0, npc_K = 0;
  uint32_t npc_edge = 0;
  int lut_shift = 0;
  uint32_t lut_base = 0;
  bool lut_one = false;            // one threshold step after the table is exact for every d^2 <= R^2
  int disjoint = 0;
  std::vector<int8_t> setidx;      // [nC][256]
};

struct Result {
  bool valid = false;
  bool batched = false;
  int nreal = 1;
  RunPlan plan;
  uint32_t nbins = 0;
  int ntasks = 0;
  std::vector<uint32_t> trg, env;  // task masks
  DevBuf rdf, knn, cnt, counters, status, npc, tests;
  uint64_t ncentres_total = 0, n_ions = 0;
  std::vector<unsigned long long> counters_h;  // per realisation [pairs, centres]
  std::vector<uint64_t> centres_sel;           // per realisation (selected count, plain runs)
  cudaStream_t stream = nullptr;
  bool fetched = false;
  std::vector<unsigned long long> rdf_h, knn_h, cnt_h;
  PinBuf stage;  // one download of status, cores and counters
};

}  // namespace

struct pp_ctx {
  int device = 0;
  int sm_count = 0;
  std::string err;
  std::vector<std::unique_ptr<Cloud>> clouds;
  std::vector<std::unique_ptr<Cloud>> spare;  // freed clouds whose device buffers later uploads reuse
  bool tasks_ok = false;
  int ntasks = 0;
  std::vector<uint32_t> trg, env;
  bool hist_ok = false;
  Tables tab;
  Result res;
  // scratch
  DevBuf tmp_cell_of, tmp_rank, scan_tmp, bbox, centres, centre_count, work, tables_dev, sel_flags, sel_tmp;
  DevBuf tri_fill, cflag, rowtab, nc_pre;
  DevBuf labels_run, perm_dev, gather_src;
  DevBuf mask_in;  // caller's centre mask: [n] input order, then [n] sorted-slot order
  // statistics after clustering: option "aposteriori_guard" = 1 runs the
  // reference's guard loop as written (see pp_run_aposteriori)
  bool apost_ref = false;
  DevBuf apost_cnt;               // neighbours within R per ion (input order)
  DevBuf multi_cmask, multi_cores;  // merged serving pass: hull-distance bits, cores + counters
  int server_batch = pp::kMultiMaxQueries;  // option "server_batch": most queries per merged pass
  uint64_t apost_relabelled = 0;  // ions the last such run relabelled
  // batched geometry cache
  DevBuf pair_count, pair_off, pair_slot, pair_cat, geo_centres, centre_ok, real_labels, rois_dev;
  DevBuf labels_il, ok_il;  // group-major interleaved copies of real_labels / centre_ok
  DevBuf knn_labels, knn_ok, knn_rec, knn_recc;  // 32-realisation kNN: layouts and records
  DevBuf knn_rest_labels, knn_rest_ok;           // the realisations after the last full 32
  DevBuf maxlist;           // longest pair list (one uint32)
  uint32_t geo_maxlist = 0;
  uint64_t geo_key_version = ~0ull;
  int geo_cloud = -1;
  float geo_R = -1.f;
  uint32_t geo_ncentres = 0;
  uint64_t geo_pairs = 0;
  bool geo_emitted_all = false;  // the pair buffer holds every list (not one chunk's)
  uint64_t pair_cap_opt = 0;     // option "batched_pair_cap": most pairs held at once (0 = by free memory)
  uint32_t npc_order = 0;        // option "npcorr_order": SpatStatKNNOrder - 1 of the n-point correlations
  DevBuf geo_counters;           // pair counters of the geometry passes
  int geo_H = 0;
  float geo_rmin = 0, geo_rincr = 0;
  uint64_t grid_counter = 1;
  bool no_sym = false;  // testing hook: force the one-sided scan
  bool no_lanes = false;  // option "lanes" = 0: RDF passes take the per-centre or brick scan
  bool no_uniform = false;  // option "uniform_sets" = 0: the kNN lane scan decodes sets per centre slot
  bool no_box = false;      // option "box_filter" = 0: the lane scans stage every candidate of the cell rows
  int knn_lists = 0;        // option "knn_lists": 0 automatic, 1 d^2 lists, 2 category lists
  DevBuf brows;           // stencil rows of a cell block, nearest first (centre-per-lane scan)
  int brows_key[3] = {-1, -1, -1};
  pp_ctx* parent = nullptr;     // serving workers share the parent's clouds
  bool readonly_clouds = false; // ... and never rebuild them
  DevBuf surf_own;              // ion2surf for an R' the cloud does not cache
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // batched apply as a CUDA graph: captured on a private stream, replayed
  // while the launch parameters (buffers, sizes, tiles) stay the same
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t apply_exec = nullptr;
  std::string apply_sig;
  uint64_t graph_nodes = 0, graph_captures = 0, graph_launches = 0;
  bool ev_recorded = false;
  int last_kind = 0;  // kernel of the last plain pass: 0 per-centre scan, 1 brick, 2/3 centre-per-lane RDF/kNN,
                      // 4/5 centre-per-lane RDF then centre-per-lane kNN / per-centre kNN
  uint64_t last_centres_all = 0;  // centres of the last plain pass before any tuning sample
};

namespace {

int fail(pp_ctx* c, int code, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? PP_ERR_NOMEM : PP_ERR_CUDA, "%s: %s", \
                  #call, cudaGetErrorString(e_));                                             \
  } while (0)

// ---------------------------------------------------------------- histogram
// Category of one float distance under histogram::add
// (src/PARAPROBE_Histogram.h:97-117): 0 lowest, 1 + b bin b, nbins + 1 highest.
int category_of_distance(const Tables& t, float x) {
  const double xx = x;
  if (xx >= t.hstart && xx <= t.hend) {
    const float rb = (float)((xx - t.hstart) * t.hscale);
    const uint32_t b = (uint32_t)std::floor(rb);
    return b < t.nbins ? (int)(1 + b) : (int)(t.nbins + 1);
  }
  if (xx < t.hstart) return 0;
  return (int)(t.nbins + 1);
}

int category_of_d2(const Tables& t, float d2) { return category_of_distance(t, std::sqrt(d2)); }

void set_tables(Tables& t, float rmin, float rincr, float rmax) {
  t.rmin = rmin; t.rincr = rincr; t.rmax = rmax;
  t.hstart = rmin; t.hend = rmax;
  size_t nb = 0;
  if ((double)rincr > kEpsilon) nb = (size_t)(((double)rmax - (double)rmin) / (double)rincr);
  t.nbins = (uint32_t)nb;
  t.hscale = nb ? 1.0 / (t.hend - t.hstart) * (double)nb : 0.0;
}

// T[k] = smallest non-negative float d^2 whose category is >= k (k = 1..H-1),
// +inf when no finite d^2 reaches k.  The category is monotone in d^2, so a
// binary search over the ordered bit patterns of non-negative floats finds it.
std::vector<float> threshold_table(const Tables& t) {
  const int H = (int)t.nbins + 2;
  std::vector<float> T(H, 0.f);
  for (int k = 1; k < H; ++k) {
    uint32_t lo = 0, hi = 0x7f800000u;  // +inf
    auto cat = [&](uint32_t u) {
      float f;
      std::memcpy(&f, &u, 4);
      return category_of_d2(t, f);
    };
    if (cat(0x7f7fffffu) < k) { T[k] = INFINITY; continue; }
    hi = 0x7f7fffffu;
    while (lo < hi) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (cat(mid) >= k) hi = mid; else lo = mid + 1;
    }
    std::memcpy(&T[k], &lo, 4);
  }
  return T;
}

// Category lookup table over the ordered bit patterns of d^2 in [0, R^2]:
// cell c covers the patterns with (bits >> shift) == base + c and holds the
// category of its smallest d^2 (cell 0 also takes every smaller d^2, all of
// category T-count-at-0).  The device starts there and steps up through T, so
// the result equals the threshold search for any shift; the shift is the
// finest that keeps the table within max_cells, so a cell rarely spans more
// than one threshold.
void build_lut(const std::vector<float>& T, float r2, int max_cells, std::vector<uint16_t>& lut, int& shift,
               uint32_t& base, bool* one_step = nullptr) {
  const int H = (int)T.size();
  auto bits = [](float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; };
  auto cat = [&](float d2) {
    int k = 0;
    while (k + 1 < H && T[k + 1] <= d2) ++k;
    return k;
  };
  float tmin = r2;
  for (int k = 1; k < H; ++k)
    if (T[k] > 0.f && T[k] < tmin) tmin = T[k];
  const uint32_t top = bits(std::max(r2, 0.f));
  for (shift = 0; shift < 31; ++shift) {
    base = bits(tmin) >> shift;
    if ((int64_t)(top >> shift) - (int64_t)base + 1 <= max_cells) break;
  }
  base = bits(tmin) >> shift;
  const int n = (int)((top >> shift) - base + 1);
  lut.assign(n, 0);
  lut[0] = (uint16_t)cat(0.f);
  for (int c = 1; c < n; ++c) {
    const uint32_t u = (base + (uint32_t)c) << shift;
    float f;
    std::memcpy(&f, &u, 4);
    lut[c] = (uint16_t)cat(f);
  }
  if (one_step) {
    // categories rise with d^2, so within cell c they run from lut[c] to at
    // most lut[c + 1] (cell 0 also takes every d^2 below it: no positive
    // threshold lies there); the last cell holds r2, and only d^2 <= r2 count
    bool one = true;
    for (int c = 0; c + 1 < n && one; ++c) one = lut[c + 1] <= lut[c] + 1;
    *one_step = one && cat(std::max(r2, 0.f)) <= lut[n - 1] + 1;
  }
}

inline bool has_type(const uint32_t* m, int t) { return (m[t >> 5] >> (t & 31)) & 1u; }

// --------------------------------------------------------------------- grid
int build_grid(pp_ctx* ctx, Cloud& cl, float R, cudaStream_t s) {
  const uint64_t n = cl.n;
  CK(ctx->bbox.ensure(8 * sizeof(uint32_t)));
  uint32_t init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(ctx->bbox.p, init, sizeof init, cudaMemcpyHostToDevice, s));
  pp::launch_bbox(cl.xyz.as<float>(), n, ctx->bbox.as<float>(), s);
  uint32_t bb[8];
  CK(cudaMemcpyAsync(bb, ctx->bbox.p, sizeof bb, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (bb[6]) return fail(ctx, PP_ERR_INVALID, "cloud has %u non-finite coordinates", bb[6]);
  auto o2f = [](uint32_t o) {
    const uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
  };
  float lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = n ? o2f(bb[k]) : 0.f;
    hi[k] = n ? o2f(bb[3 + k]) : 0.f;
  }
  // cell edge R / cell_ratio (3 by default, tuned by pp_autotune), coarsened
  // if the grid would hold more than max(4 n, 2^20) cells
  double h = std::max((double)R / std::max(cl.cell_ratio, 0.5f), 1e-3);
  const double ext[3] = {(double)hi[0] - lo[0], (double)hi[1] - lo[1], (double)hi[2] - lo[2]};
  const double maxcells = std::max(4.0 * (double)n, (double)(1 << 20));
  for (;;) {
    double c = 1.0;
    for (int k = 0; k < 3; ++k) c *= std::floor(ext[k] / h) + 1.0;
    if (c <= maxcells && c < 4.0e9) break;
    h *= 1.25;
  }
  Grid g{};
  g.h = (float)h;
  g.inv_h = (float)(1.0 / h);
  g.lox = lo[0]; g.loy = lo[1]; g.loz = lo[2];
  g.nx = (int)std::floor(ext[0] / h) + 1;
  g.ny = (int)std::floor(ext[1] / h) + 1;
  g.nz = (int)std::floor(ext[2] / h) + 1;
  g.ncells = (uint64_t)g.nx * g.ny * g.nz;
  const double amax = std::max({std::fabs((double)lo[0]), std::fabs((double)hi[0]), std::fabs((double)lo[1]),
                                std::fabs((double)hi[1]), std::fabs((double)lo[2]), std::fabs((double)hi[2])});
  g.margin = (float)std::max(1e-3 * h, 1e-5 * amax + 1e-6);

  CK(ctx->tmp_cell_of.ensure(n * 4));
  CK(ctx->tmp_rank.ensure(n * 4));
  CK(cl.cell_start.ensure((g.ncells + 1) * 4));
  CK(cudaMemsetAsync(cl.cell_start.p, 0, (g.ncells + 1) * 4, s));
  pp::launch_cell_count(cl.xyz.as<float>(), n, g, ctx->tmp_cell_of.as<uint32_t>(), ctx->tmp_rank.as<uint32_t>(),
                        cl.cell_start.as<uint32_t>(), s);
  const uint64_t tmp_elems = (g.ncells + 1) / 2048 + 64;
  CK(ctx->scan_tmp.ensure(tmp_elems * 8 * 2));
  pp::launch_exclusive_scan_u32(cl.cell_start.as<uint32_t>(), g.ncells + 1, ctx->scan_tmp.as<uint32_t>(),
                                tmp_elems * 4, s);
  CK(cl.ions.ensure(std::max<uint64_t>(n, 1) * 16));
  CK(cl.slot_of_id.ensure(std::max<uint64_t>(n, 1) * 4));
  CK(cl.id_of_slot.ensure(std::max<uint64_t>(n, 1) * 4));
  CK(cl.label_sorted.ensure(std::max<uint64_t>(n, 1)));
  pp::launch_scatter(cl.xyz.as<float>(), cl.label.as<uint8_t>(), n, ctx->tmp_cell_of.as<uint32_t>(),
                     ctx->tmp_rank.as<uint32_t>(), cl.cell_start.as<uint32_t>(), cl.ions.as<float4>(),
                     cl.slot_of_id.as<uint32_t>(), cl.id_of_slot.as<uint32_t>(), cl.label_sorted.as<uint8_t>(), s);
  CK(cudaGetLastError());
  // non-empty cells: the default cell block of the centre-per-lane scans
  unsigned long long occ = 0;
  CK(ctx->work.ensure(16));
  CK(cudaMemsetAsync(ctx->work.p, 0, 8, s));
  pp::launch_count_occupied(cl.cell_start.as<uint32_t>(), g.ncells, ctx->work.as<unsigned long long>(),
                            ctx->sm_count, s);
  CK(cudaMemcpyAsync(&occ, ctx->work.p, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  cl.occupied = occ;
  cl.g = g;
  cl.grid_ok = true;
  cl.grid_version = ctx->grid_counter++;
  return PP_OK;
}

// Default cell block of the centre-per-lane scans: about 24 centres (a warp's
// worth) at the mean number of centres per non-empty cell, twice as long in x
// as in y and z.  Returns false when centres are too sparse for a block to
// fill a warp without streaming far more ions than the centres' balls hold
// (fewer than 0.35 centres per non-empty cell); such passes take the
// per-centre scan.
bool default_block(const Cloud& cl, uint64_t ncent, int* bx, int* by, int* bz) {
  const double per_cell = cl.occupied ? (double)ncent / (double)cl.occupied : 0.0;
  if (per_cell < 0.35) return false;
  const double cells = std::max(1.0, 24.0 / per_cell);
  const int side = (int)std::lround(std::cbrt(cells / 2.0));
  *by = *bz = std::min(15, std::max(1, side));
  *bx = (int)std::min(64L, std::max(1L, std::lround(cells / ((double)*by * *bz))));
  return true;
}

// A grid serves every radius with R / h in [1, 6] (stencils of 3..13 cells a
// side); outside that range it is rebuilt with h = R / cell_ratio.  Contexts
// that share a parent's clouds (serving workers) may not rebuild.
int ensure_grid(pp_ctx* ctx, Cloud& cl, float R, cudaStream_t s) {
  if (cl.grid_ok && cl.g.h <= R * 1.0001f && cl.g.h >= R / 6.f) return PP_OK;
  if (ctx->readonly_clouds)
    return fail(ctx, PP_ERR_STATE, "cloud was not prepared for R = %g (pp_cloud_prepare)", (double)R);
  return build_grid(ctx, cl, R, s);
}

// ------------------------------------------------------------- ion2surf
// Triangle boxes (fmin/fmax of the vertices, src/PARAPROBE_SolverHdl.cpp:
// 2712-2717) and per-cell triangle lists of a hull grid.  A triangle is listed
// in every cell its box grown by `grow` reaches, so the lists serve every
// query radius R' with R' + slack <= grow.  The hull grid is the cloud's ion
// grid coarsened f times per axis (f ~ R' / h), so it is rebuilt with the ion
// grid and the hull distance walks each hull cell's ions as whole rows.
int ensure_tri_bins(pp_ctx* ctx, Cloud& cl, float rp, cudaStream_t s) {
  if (cl.tri_ok && cl.tri_grow >= rp + cl.tri_slack && cl.tri_grid_version == cl.grid_version) return PP_OK;
  const std::vector<float>& tri = cl.hull.tri;
  const uint64_t nt = tri.size() / 9;
  // the hull's bounds were taken at upload; the boxes are built on the device
  float glo[3] = {cl.hull.lo[0], cl.hull.lo[1], cl.hull.lo[2]}, ghi[3] = {cl.hull.hi[0], cl.hull.hi[1], cl.hull.hi[2]};
  // slack: float rounding of cell indices, of the hull's and of the ions'
  // coordinates (the ion grid's margin)
  const float slack = std::max(1e-3f + 1e-5f * std::max({std::fabs(glo[0]), std::fabs(ghi[0]), std::fabs(glo[1]),
                                                         std::fabs(ghi[1]), std::fabs(glo[2]), std::fabs(ghi[2])}),
                               cl.grid_ok ? 2.f * cl.g.margin : 0.f);
  const float grow = rp + slack;
  if (cl.tri_ok && cl.tri_grow >= grow && cl.tri_grid_version == cl.grid_version) return PP_OK;
  if (ctx->readonly_clouds)
    return fail(ctx, PP_ERR_STATE, "hull lists were not prepared for R' = %g (pp_cloud_prepare)", (double)rp);
  if (!cl.grid_ok) return fail(ctx, PP_ERR_STATE, "hull lists need the cloud's grid");
  const Grid& g = cl.g;
  int f = std::max(1, (int)std::lround((double)rp / (double)g.h));
  auto hull_cells = [&](int ff) {
    return (uint64_t)((g.nx + ff - 1) / ff) * (uint64_t)((g.ny + ff - 1) / ff) * (uint64_t)((g.nz + ff - 1) / ff);
  };
  while (hull_cells(f) >= 60000000ull) ++f;
  Grid tg{};
  tg.h = g.h * (float)f;
  tg.inv_h = (float)(1.0 / ((double)g.h * f));
  tg.lox = g.lox; tg.loy = g.loy; tg.loz = g.loz;
  tg.nx = (g.nx + f - 1) / f;
  tg.ny = (g.ny + f - 1) / f;
  tg.nz = (g.nz + f - 1) / f;
  tg.ncells = hull_cells(f);
  CK(cl.tri_dev.ensure(std::max<size_t>(tri.size(), 1) * 4));
  CK(cudaMemcpyAsync(cl.tri_dev.p, tri.data(), tri.size() * 4, cudaMemcpyHostToDevice, s));
  CK(cl.tri_box.ensure(std::max<size_t>(6 * nt, 1) * 4));
  if (nt) pp::launch_tri_box(cl.tri_dev.as<float>(), nt, cl.tri_box.as<float>(), s);
  CK(cl.tcell_start.ensure((tg.ncells + 1) * 4));
  CK(ctx->tri_fill.ensure((tg.ncells + 1) * 4));
  const uint64_t tmp_elems = (tg.ncells + 1) / 2048 + 64;
  CK(ctx->scan_tmp.ensure(tmp_elems * 8 * 2));
  uint64_t total = 0;
  uint64_t cap = cl.tcell_list.bytes / 4;
  int brc = pp::launch_tri_bins(cl.tri_box.as<float>(), nt, tg, grow, cl.tcell_start.as<uint32_t>(),
                                ctx->tri_fill.as<uint32_t>(), cl.tcell_list.as<uint32_t>(), cap,
                                ctx->scan_tmp.as<uint32_t>(), tmp_elems * 4, &total, s);
  if (brc == 1) {
    CK(cl.tcell_list.ensure(std::max<uint64_t>(total, 1) * 4));
    cap = cl.tcell_list.bytes / 4;
    brc = pp::launch_tri_bins(cl.tri_box.as<float>(), nt, tg, grow, cl.tcell_start.as<uint32_t>(),
                              ctx->tri_fill.as<uint32_t>(), cl.tcell_list.as<uint32_t>(), cap,
                              ctx->scan_tmp.as<uint32_t>(), tmp_elems * 4, &total, s);
  }
  if (brc) return fail(ctx, PP_ERR_CUDA, "triangle binning failed");
  CK(cudaStreamSynchronize(s));  // the triangles were copied from the cloud's host vector
  cl.tg = tg;
  cl.tri_f = f;
  cl.tri_grid_version = cl.grid_version;
  cl.tri_grow = grow;
  cl.tri_slack = slack;
  cl.tri_ok = true;
  return PP_OK;
}

// ion2surf of the run in sorted-slot order: from the caller's values, or R'^2
// without a hull (src/PARAPROBE_SolverHdl.cpp:335-348), or computed against
// the hull with R' = max(R, SurfaceCellsCarvingRadius).  The cloud caches one
// R'; a serving worker computes other R' into its own buffer.
int ensure_surface(pp_ctx* ctx, Cloud& cl, float R, cudaStream_t s, const float** surf_out) {
  const uint64_t n = cl.n;
  if (cl.has_user_surf) {
    if (!(cl.surf_version == cl.grid_version && cl.surf_rp < 0.f)) {
      if (ctx->readonly_clouds) return fail(ctx, PP_ERR_STATE, "cloud was not prepared (pp_cloud_prepare)");
      CK(cl.surf.ensure(std::max<uint64_t>(n, 1) * 4));
      pp_host::gather_f32_sorted(cl.user_surf.as<float>(), cl.id_of_slot.as<uint32_t>(), n, cl.surf.as<float>(), s);
      cl.surf_rp = -1.f;
      cl.surf_version = cl.grid_version;
    }
    *surf_out = cl.surf.as<float>();
    return PP_OK;
  }
  const float rp = std::max(R, cl.hull.carve);  // max(SpatStatRadiusMax, SurfaceCellsCarvingRadius)
  if (cl.surf_version == cl.grid_version && cl.surf_rp == rp) {
    *surf_out = cl.surf.as<float>();
    return PP_OK;
  }
  DevBuf* dst = &cl.surf;
  if (ctx->readonly_clouds) dst = &ctx->surf_own;
  CK(dst->ensure(std::max<uint64_t>(n, 1) * 4));
  if (!cl.hull.present) {
    pp_host::fill_f32(dst->as<float>(), n, rp * rp, s);
  } else {
    int rc = ensure_tri_bins(ctx, cl, rp, s);
    if (rc) return rc;
    pp::launch_surface_cells(cl.ions.as<float4>(), cl.cell_start.as<uint32_t>(), cl.g, cl.tri_f,
                             cl.tri_box.as<float>(), cl.tri_dev.as<float>(), cl.tcell_start.as<uint32_t>(),
                             cl.tcell_list.as<uint32_t>(), cl.tg, rp, dst->as<float>(), s);
    CK(cudaGetLastError());
  }
  if (!ctx->readonly_clouds) {
    cl.surf_rp = rp;
    cl.surf_version = cl.grid_version;
  }
  *surf_out = dst->as<float>();
  return PP_OK;
}

// ------------------------------------------------------------------- plan
int make_plan(pp_ctx* ctx, uint32_t flags, const uint32_t* k_list, int nk, RunPlan& P) {
  if (!ctx->tasks_ok) return fail(ctx, PP_ERR_STATE, "pp_tasks_set was not called");
  if (!ctx->hist_ok) return fail(ctx, PP_ERR_STATE, "pp_hist_params was not called");
  if (flags & ~(PP_RDF | PP_1NN | PP_RIPK | PP_MKNN | PP_CNTNB | PP_NPCORR)) return fail(ctx, PP_ERR_INVALID, "unknown flags");
  const Tables& t = ctx->tab;
  if (t.nbins == 0) return fail(ctx, PP_ERR_INVALID, "histogram has no bins (rincr <= 1e-6 or rmax <= rmin)");
  if (t.nbins + 2 > 16384) return fail(ctx, PP_ERR_UNSUPPORTED, "more than 16382 bins");
  P = RunPlan();
  P.flags = flags;
  P.H = (int)t.nbins + 2;
  if ((flags & PP_MKNN) && nk > 0) {
    if (!k_list) return fail(ctx, PP_ERR_INVALID, "k_list is NULL");
    for (int i = 0; i < nk; ++i) {
      if (k_list[i] < 1) return fail(ctx, PP_ERR_INVALID, "k order smaller than 1");
      P.k_out.push_back(k_list[i]);
    }
  }
  std::vector<uint32_t> ks = P.k_out;
  if (flags & PP_1NN) ks.push_back(1);
  std::sort(ks.begin(), ks.end());
  ks.erase(std::unique(ks.begin(), ks.end()), ks.end());
  P.kvals = ks;
  P.kmax = ks.empty() ? 0 : (int)ks.back();
  if (P.kmax > 128) return fail(ctx, PP_ERR_UNSUPPORTED, "k = %d exceeds the register-resident limit of 128", P.kmax);
  P.kr = P.kmax == 0 ? 0 : (P.kmax <= 32 ? 1 : 4);
  // type slots
  const int nt = ctx->ntasks;
  P.cslot_of.assign(256, -1);
  P.eslot_of.assign(256, -1);
  for (int ty = 0; ty < 256; ++ty) {
    bool c = false, e = false;
    for (int k = 0; k < nt; ++k) {
      c |= has_type(&ctx->trg[8 * k], ty);
      e |= has_type(&ctx->env[8 * k], ty);
    }
    if (c) { P.cslot_of[ty] = (int8_t)P.ctype.size(); P.ctype.push_back(ty); }
    if (e) { P.eslot_of[ty] = (int8_t)P.etype.size(); P.etype.push_back(ty); }
  }
  if (P.ctype.size() > 127 || P.etype.size() > 127) return fail(ctx, PP_ERR_UNSUPPORTED, "more than 127 distinct types in tasks");
  P.nC = (int)P.ctype.size();
  P.nE = (int)P.etype.size();
  // distinct environment sets
  std::map<std::vector<uint32_t>, int> setid;
  P.task_set.assign(nt, -1);
  for (int k = 0; k < nt; ++k) {
    std::vector<uint32_t> m(&ctx->env[8 * k], &ctx->env[8 * k] + 8);
    auto it = setid.find(m);
    if (it == setid.end()) { it = setid.emplace(m, (int)P.sets.size()).first; P.sets.push_back(m); }
    P.task_set[k] = it->second;
  }
  P.nS = (int)P.sets.size();
  P.envbits.assign((size_t)std::max(P.nC, 1) * 256, 0u);
  P.set_list.assign((size_t)std::max(P.nC, 1) * 32, -1);
  P.nsets.assign(std::max(P.nC, 1), 0);
  for (int c = 0; c < P.nC; ++c) {
    std::vector<int> local;
    for (int k = 0; k < nt; ++k) {
      if (!has_type(&ctx->trg[8 * k], P.ctype[c])) continue;
      if (std::find(local.begin(), local.end(), P.task_set[k]) == local.end()) local.push_back(P.task_set[k]);
    }
    if ((P.kr > 0 || (flags & PP_NPCORR)) && local.size() > 32)
      return fail(ctx, PP_ERR_UNSUPPORTED, "more than 32 environment sets for one centre type");
    P.nsets[c] = (int)local.size();
    for (size_t p = 0; p < local.size() && p < 32; ++p) {
      P.set_list[c * 32 + p] = local[p];
      for (int ty = 0; ty < 256; ++ty)
        if (has_type(P.sets[local[p]].data(), ty)) P.envbits[c * 256 + ty] |= (1u << p);
    }
    P.emax = std::max(P.emax, (int)local.size());
  }
  if (P.kr == 4 && P.emax > 8) return fail(ctx, PP_ERR_UNSUPPORTED, "k > 32 with more than 8 environment sets per centre type");
  // disjoint sets: no type in two environment sets of one centre type (the
  // usual "A-B" task lists); then a type names its set directly
  P.disjoint = 1;
  P.setidx.assign((size_t)std::max(P.nC, 1) * 256, (int8_t)-1);
  for (int c = 0; c < P.nC; ++c)
    for (int ty = 0; ty < 256; ++ty) {
      const uint32_t b = P.envbits[c * 256 + ty];
      if (__builtin_popcount(b) > 1) P.disjoint = 0;
      if (b) P.setidx[c * 256 + ty] = (int8_t)__builtin_ctz(b);
    }
  if (flags & PP_NPCORR) {
    // npc3d geometry (src/PARAPROBE_NPointCorrelations3D.cpp:53-73) and the
    // size limit of src/PARAPROBE_SolverHdl.cpp:3706-3712
    const float realhalf = std::ceil(t.rmax / t.rincr) + 1.f;
    P.npc_half = (int)realhalf;
    P.npc_edge = 1u + 2u * (uint32_t)P.npc_half;
    const double nxyz = (double)P.npc_edge * P.npc_edge * P.npc_edge;
    if (nxyz > 503.0 * 503.0 * 503.0)
      return fail(ctx, PP_ERR_UNSUPPORTED, "Computation of 2-point statistics would require too large buffers");
    P.npc_K = (int)ctx->npc_order + 1;
    P.ntk.assign(std::max(P.nC, 1), 0);
    P.tk_task.assign((size_t)std::max(P.nC, 1) * 32, -1);
    P.tk_set.assign((size_t)std::max(P.nC, 1) * 32, -1);
    for (int c = 0; c < P.nC; ++c)
      for (int k = 0; k < nt; ++k) {
        if (!has_type(&ctx->trg[8 * k], P.ctype[c])) continue;
        if (P.ntk[c] == 32) return fail(ctx, PP_ERR_UNSUPPORTED, "more than 32 n-point correlation tasks per centre type");
        int q = 0;
        while (q < P.nsets[c] && P.set_list[c * 32 + q] != P.task_set[k]) ++q;
        P.tk_task[c * 32 + P.ntk[c]] = k;
        P.tk_set[c * 32 + P.ntk[c]] = q;
        ++P.ntk[c];
      }
  }
  P.catT = threshold_table(t);
  build_lut(P.catT, t.rmax * t.rmax, 4096, P.lut, P.lut_shift, P.lut_base, &P.lut_one);
  P.cat_miss = category_of_distance(t, (float)((double)t.rmax + kEpsilon));
  return PP_OK;
}

// Upload the plan's tables into one device block; returns device pointers.
struct DevTables {
  float* catT; int8_t* cslot; int8_t* eslot; uint32_t* envbits; int* set_list; int* nsets; int* kvals;
  uint16_t* lut;
  int8_t* setidx;
  int8_t* rowtab;
  int* ntk; int* tk_task; int* tk_set;
};

int upload_tables(pp_ctx* ctx, const RunPlan& P, DevTables& D, cudaStream_t s) {
  std::vector<unsigned char> blob;
  auto put = [&](const void* src, size_t bytes) {
    size_t off = (blob.size() + 15) & ~size_t(15);
    blob.resize(off + bytes);
    if (bytes) std::memcpy(blob.data() + off, src, bytes);
    return off;
  };
  const size_t o1 = put(P.catT.data(), P.catT.size() * 4);
  const size_t o2 = put(P.cslot_of.data(), 256);
  const size_t o3 = put(P.eslot_of.data(), 256);
  const size_t o4 = put(P.envbits.data(), P.envbits.size() * 4);
  const size_t o5 = put(P.set_list.data(), P.set_list.size() * 4);
  const size_t o6 = put(P.nsets.data(), P.nsets.size() * 4);
  std::vector<int> kv(P.kvals.begin(), P.kvals.end());
  if (kv.empty()) kv.push_back(1);
  const size_t o7 = put(kv.data(), kv.size() * 4);
  const size_t o8 = put(P.setidx.data(), P.setidx.size());
  int nrow = 0;
  const int8_t* rows = pp::row_table_host(&nrow);
  const size_t o9 = put(rows, (size_t)nrow * 2);
  const size_t o10 = put(P.lut.data(), P.lut.size() * 2);
  const size_t o11 = put(P.ntk.data(), P.ntk.size() * 4);
  const size_t o12 = put(P.tk_task.data(), P.tk_task.size() * 4);
  const size_t o13 = put(P.tk_set.data(), P.tk_set.size() * 4);
  CK(ctx->tables_dev.ensure(blob.size()));
  CK(cudaMemcpyAsync(ctx->tables_dev.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));  // blob is a host temporary
  unsigned char* b = ctx->tables_dev.as<unsigned char>();
  D.catT = (float*)(b + o1); D.cslot = (int8_t*)(b + o2); D.eslot = (int8_t*)(b + o3);
  D.envbits = (uint32_t*)(b + o4); D.set_list = (int*)(b + o5); D.nsets = (int*)(b + o6); D.kvals = (int*)(b + o7);
  D.setidx = (int8_t*)(b + o8);
  D.rowtab = (int8_t*)(b + o9);
  D.lut = (uint16_t*)(b + o10);
  D.ntk = (int*)(b + o11);
  D.tk_task = (int*)(b + o12);
  D.tk_set = (int*)(b + o13);
  return PP_OK;
}

Cloud* get_cloud(pp_ctx* ctx, int id) {
  std::vector<std::unique_ptr<Cloud>>& v = ctx->parent ? ctx->parent->clouds : ctx->clouds;
  if (id < 0 || id >= (int)v.size()) return nullptr;
  return v[id].get();
}

void fill_scan_common(pp::ScanArgs& a, const Cloud& cl, const RunPlan& P, const DevTables& D, const Tables& t) {
  a.ions = cl.ions.as<float4>();
  a.cell_start = cl.cell_start.as<uint32_t>();
  a.g = cl.g;
  a.R = t.rmax;
  a.R2 = t.rmax * t.rmax;
  a.box_R2 = std::nextafter(a.R2 * (1.f + 1.f / 4096.f) + 1e-30f, std::numeric_limits<float>::infinity());
  a.no_box_filter = 0;
  const float Rm = t.rmax + cl.g.margin;
  a.Rm2 = Rm * Rm;
  a.H = P.H;
  a.cat_T = D.catT;
  a.guess_start = t.rmin;
  a.guess_scale = (float)t.hscale;
  a.cat_lut = D.lut;
  a.lut_n = (int)P.lut.size();
  a.lut_shift = P.lut_shift;
  a.lut_base = P.lut_base;
  a.lut_one = P.lut_one ? 1 : 0;
  a.cat_miss = P.cat_miss;
  a.cslot_of = D.cslot;
  a.eslot_of = D.eslot;
  a.nC = P.nC;
  a.nE = P.nE;
  a.envbits = D.envbits;
  a.set_list = D.set_list;
  a.nsets = D.nsets;
  a.nS = P.nS;
  a.kvals = D.kvals;
  a.nkI = (int)P.kvals.size();
  a.kmax = std::max(P.kmax, 1);
  // shared-memory kNN lists when every type names one set and they fit
  a.disjoint = (P.disjoint && (size_t)8 * std::max(P.emax, 1) * (P.kr * 32 + 1) * 4 <= 64 * 1024) ? 1 : 0;
  a.emax = std::max(P.emax, 1);
  a.setidx = D.setidx;
  a.uniform_sets = 1;
  for (int c = 1; c < P.nC && a.uniform_sets; ++c)
    if (std::memcmp(&P.setidx[(size_t)c * 256], &P.setidx[0], 256) != 0) a.uniform_sets = 0;
  a.tile = std::max<uint32_t>(cl.tile, 1);
  a.rowtab = D.rowtab;
  a.sym = 0;
}

// Fold per-type cores into per-task histograms (pp_fetch layout).
void finalize(const Result& R, int r, uint64_t* out) {
  const RunPlan& P = R.plan;
  const int H = P.H, nt = R.ntasks;
  const size_t rdf_sz = (size_t)P.nC * P.nE * H;
  const size_t knn_sz = (size_t)P.nC * P.nS * P.kvals.size() * H;
  const unsigned long long* rdf = R.rdf_h.data() + (size_t)r * rdf_sz;
  const unsigned long long* knn = R.knn_h.empty() ? nullptr : R.knn_h.data() + (size_t)r * knn_sz;
  uint64_t o = 0;
  auto kidx = [&](uint32_t k) { return (int)(std::lower_bound(P.kvals.begin(), P.kvals.end(), k) - P.kvals.begin()); };
  // a task's histogram is the sum of the per-type cores it covers: the cores
  // are listed once per task, then added bin row by bin row
  std::vector<const unsigned long long*> rows;
  auto add_rows = [&]() {
    uint64_t* dst = out + o;
    std::fill(dst, dst + H, 0ull);
    for (const unsigned long long* src : rows)
      for (int b = 0; b < H; ++b) dst[b] += src[b];
    o += (uint64_t)H;
  };
  auto rdf_task = [&](int t) {
    rows.clear();
    for (int c = 0; c < P.nC; ++c) {
      if (!has_type(&R.trg[8 * t], P.ctype[c])) continue;
      for (int e = 0; e < P.nE; ++e)
        if (has_type(&R.env[8 * t], P.etype[e])) rows.push_back(rdf + ((size_t)c * P.nE + e) * H);
    }
    add_rows();
  };
  auto knn_task = [&](int t, int ki) {
    const int Sg = P.task_set[t];
    rows.clear();
    for (int c = 0; c < P.nC; ++c)
      if (has_type(&R.trg[8 * t], P.ctype[c])) rows.push_back(knn + (((size_t)c * P.nS + Sg) * P.kvals.size() + ki) * H);
    add_rows();
  };
  if (P.flags & PP_RDF) for (int t = 0; t < nt; ++t) rdf_task(t);
  if (P.flags & PP_1NN) for (int t = 0; t < nt; ++t) knn_task(t, kidx(1));
  if (P.flags & PP_RIPK) for (int t = 0; t < nt; ++t) rdf_task(t);
  if ((P.flags & PP_MKNN) && !P.k_out.empty())
    for (int t = 0; t < nt; ++t)
      for (uint32_t k : P.k_out) knn_task(t, kidx(k));
}

uint64_t result_len(const Result& R) {
  const RunPlan& P = R.plan;
  uint64_t g = 0;
  if (P.flags & PP_RDF) g += R.ntasks;
  if (P.flags & PP_1NN) g += R.ntasks;
  if (P.flags & PP_RIPK) g += R.ntasks;
  if (P.flags & PP_MKNN) g += (uint64_t)R.ntasks * P.k_out.size();
  return g * P.H;
}

int fetch_cores(pp_ctx* ctx) {
  Result& R = ctx->res;
  if (!R.valid) return fail(ctx, PP_ERR_STATE, "no run to fetch");
  if (R.fetched) return PP_OK;
  const RunPlan& P = R.plan;
  const size_t rdf_sz = (P.flags & (PP_RDF | PP_RIPK)) ? (size_t)P.nC * P.nE * P.H * R.nreal : 0;
  const size_t knn_sz = P.kr ? (size_t)P.nC * P.nS * P.kvals.size() * P.H * R.nreal : 0;
  const size_t cnt_sz = ((P.flags & PP_CNTNB) && !R.batched) ? (size_t)P.nC * P.nE * (P.cmax + 1) : 0;
  const size_t ctr_sz = 2 * (size_t)R.nreal;
  // everything through one page-locked buffer: [status pad] [counters] [rdf] [knn] [cnt]
  CK(R.stage.ensure(8 * (1 + ctr_sz + rdf_sz + knn_sz + cnt_sz)));
  unsigned long long* h = static_cast<unsigned long long*>(R.stage.p);
  CK(cudaMemcpyAsync(h, R.status.p, 4, cudaMemcpyDeviceToHost, R.stream));
  CK(cudaMemcpyAsync(h + 1, R.counters.p, 8 * ctr_sz, cudaMemcpyDeviceToHost, R.stream));
  if (rdf_sz) CK(cudaMemcpyAsync(h + 1 + ctr_sz, R.rdf.p, 8 * rdf_sz, cudaMemcpyDeviceToHost, R.stream));
  if (knn_sz) CK(cudaMemcpyAsync(h + 1 + ctr_sz + rdf_sz, R.knn.p, 8 * knn_sz, cudaMemcpyDeviceToHost, R.stream));
  if (cnt_sz)
    CK(cudaMemcpyAsync(h + 1 + ctr_sz + rdf_sz + knn_sz, R.cnt.p, 8 * cnt_sz, cudaMemcpyDeviceToHost, R.stream));
  CK(cudaStreamSynchronize(R.stream));
  int status = 0;
  std::memcpy(&status, h, 4);
  R.counters_h.assign(h + 1, h + 1 + ctr_sz);
  // finalize indexes the RDF cores whenever the plan has RDF bins
  R.rdf_h.assign((size_t)P.nC * P.nE * P.H * R.nreal, 0);
  if (rdf_sz) std::memcpy(R.rdf_h.data(), h + 1 + ctr_sz, 8 * rdf_sz);
  R.knn_h.assign(h + 1 + ctr_sz + rdf_sz, h + 1 + ctr_sz + rdf_sz + knn_sz);
  if (cnt_sz) R.cnt_h.assign(h + 1 + ctr_sz + rdf_sz + knn_sz, h + 1 + ctr_sz + rdf_sz + knn_sz + cnt_sz);
  R.fetched = true;
  if (status & pp::ST_CNT_OVERFLOW) return fail(ctx, PP_ERR_OVERFLOW, "a neighbour count exceeded the CNTNB capacity");
  if (status & pp::ST_LIST_OVERFLOW) return fail(ctx, PP_ERR_OVERFLOW, "a pair list exceeded its allocation");
  if (status) return fail(ctx, PP_ERR_DEVICE, "device status word 0x%x", status);
  return PP_OK;
}

int alloc_result(pp_ctx* ctx, const RunPlan& P, int nreal, bool batched, cudaStream_t s) {
  Result& R = ctx->res;
  R.valid = false;
  R.fetched = false;
  R.plan = P;
  R.nreal = nreal;
  R.batched = batched;
  R.ntasks = ctx->ntasks;
  R.trg = ctx->trg;
  R.env = ctx->env;
  R.nbins = ctx->tab.nbins;
  R.stream = s;
  const size_t rdf_sz = std::max<size_t>((size_t)P.nC * P.nE * P.H * nreal, 1);
  const size_t knn_sz = std::max<size_t>((size_t)P.nC * P.nS * std::max<size_t>(P.kvals.size(), 1) * P.H * nreal, 1);
  const size_t cnt_sz = std::max<size_t>((size_t)P.nC * P.nE * (P.cmax + 1), 1);
  CK(R.rdf.ensure(rdf_sz * 8));
  CK(cudaMemsetAsync(R.rdf.p, 0, rdf_sz * 8, s));
  if (P.kr) {
    CK(R.knn.ensure(knn_sz * 8));
    CK(cudaMemsetAsync(R.knn.p, 0, knn_sz * 8, s));
  }
  if (P.flags & PP_CNTNB) {
    CK(R.cnt.ensure(cnt_sz * 8));
    CK(cudaMemsetAsync(R.cnt.p, 0, cnt_sz * 8, s));
  }
  if (P.flags & PP_NPCORR) {
    const size_t npc_sz = std::max<size_t>((size_t)ctx->ntasks * P.npc_edge * P.npc_edge * P.npc_edge, 1);
    CK(R.npc.ensure(npc_sz * 4));
    CK(cudaMemsetAsync(R.npc.p, 0, npc_sz * 4, s));
  }
  CK(R.counters.ensure(16 * (size_t)nreal));
  CK(cudaMemsetAsync(R.counters.p, 0, 16 * (size_t)nreal, s));
  CK(R.status.ensure(4));
  CK(cudaMemsetAsync(R.status.p, 0, 4, s));
  return PP_OK;
}

}  // namespace

// =================================================================== C ABI
extern "C" {

const char* pp_strerror(int code) {
  switch (code) {
    case PP_OK: return "ok";
    case PP_ERR_INVALID: return "invalid argument";
    case PP_ERR_CUDA: return "CUDA error";
    case PP_ERR_NOMEM: return "out of memory";
    case PP_ERR_UNSUPPORTED: return "unsupported";
    case PP_ERR_STATE: return "call order violated";
    case PP_ERR_OVERFLOW: return "capacity exceeded";
    case PP_ERR_DEVICE: return "device reported a failure";
    case PP_ERR_IO: return "file error";
    default: return "unknown error";
  }
}

const char* pp_last_error(pp_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int pp_create(pp_ctx** out, int device) {
  if (!out) return PP_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PP_ERR_CUDA;
  if (device < 0 || device >= ndev) return PP_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return PP_ERR_CUDA;
  pp_ctx* c = new (std::nothrow) pp_ctx();
  if (!c) return PP_ERR_NOMEM;
  c->device = device;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    delete c;
    return PP_ERR_CUDA;
  }
  *out = c;
  return PP_OK;
}

void pp_destroy(pp_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->apply_exec) cudaGraphExecDestroy(ctx->apply_exec);
  if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
  delete ctx;
}

int pp_device_info(pp_ctx* ctx, int* device, int* sm_count) {
  if (!ctx) return PP_ERR_INVALID;
  if (device) *device = ctx->device;
  if (sm_count) *sm_count = ctx->sm_count;
  return PP_OK;
}

// A new cloud takes the device buffers of a freed one when one is kept
// (pp_cloud_free), so that upload-run-free loops do not pay cudaMalloc /
// cudaFree (which synchronises the device) on every cloud.
static void adopt_buffers(Cloud& to, Cloud& from) {
  DevBuf* a[] = {&to.xyz, &to.label, &to.ions, &to.cell_start, &to.slot_of_id, &to.id_of_slot, &to.label_sorted,
                 &to.user_surf, &to.surf, &to.tri_dev, &to.tri_box, &to.tcell_start, &to.tcell_list};
  DevBuf* b[] = {&from.xyz, &from.label, &from.ions, &from.cell_start, &from.slot_of_id, &from.id_of_slot,
                 &from.label_sorted, &from.user_surf, &from.surf, &from.tri_dev, &from.tri_box, &from.tcell_start,
                 &from.tcell_list};
  for (size_t i = 0; i < sizeof a / sizeof a[0]; ++i) {
    std::swap(a[i]->p, b[i]->p);
    std::swap(a[i]->bytes, b[i]->bytes);
  }
}

static int new_cloud(pp_ctx* ctx, uint64_t n, int* cloud, Cloud** out) {
  if (n > 0xfffffff0ull) return fail(ctx, PP_ERR_UNSUPPORTED, "clouds are limited to 2^32-16 ions");
  auto c = std::make_unique<Cloud>();
  if (!ctx->spare.empty()) {
    // the kept buffers that fit this cloud best: the largest position buffer
    size_t best = 0;
    for (size_t i = 1; i < ctx->spare.size(); ++i)
      if (ctx->spare[i]->xyz.bytes > ctx->spare[best]->xyz.bytes) best = i;
    adopt_buffers(*c, *ctx->spare[best]);
    ctx->spare.erase(ctx->spare.begin() + (long)best);
  }
  c->n = n;
  CK(c->xyz.ensure(std::max<uint64_t>(n, 1) * 12));
  CK(c->label.ensure(std::max<uint64_t>(n, 1)));
  *out = c.get();
  ctx->clouds.push_back(std::move(c));
  *cloud = (int)ctx->clouds.size() - 1;
  return PP_OK;
}

int pp_cloud_upload(pp_ctx* ctx, const float* xyz, const uint8_t* label, const uint32_t* ion_id, uint64_t n,
                    int* cloud) {
  if (!ctx || !cloud || (n && (!xyz || !label))) return fail(ctx, PP_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  Cloud* c = nullptr;
  int rc = new_cloud(ctx, n, cloud, &c);
  if (rc) return rc;
  CK(cudaMemcpy(c->xyz.p, xyz, n * 12, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->label.p, label, n, cudaMemcpyHostToDevice));
  if (ion_id) c->ids.assign(ion_id, ion_id + n);
  return PP_OK;
}

int pp_cloud_upload_device(pp_ctx* ctx, const float* d_xyz, const uint8_t* d_label, uint64_t n, int* cloud,
                           void* stream) {
  if (!ctx || !cloud || (n && (!d_xyz || !d_label))) return fail(ctx, PP_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  Cloud* c = nullptr;
  int rc = new_cloud(ctx, n, cloud, &c);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(c->xyz.p, d_xyz, n * 12, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(c->label.p, d_label, n, cudaMemcpyDeviceToDevice, s));
  return PP_OK;
}

int pp_cloud_upload_pos(pp_ctx* ctx, const void* pos_bytes, uint64_t n, const float* range_lo, const float* range_hi,
                        const uint8_t* range_type, int nranges, int* cloud) {
  if (!ctx || !cloud || (n && !pos_bytes) || nranges < 0 || (nranges && (!range_lo || !range_hi || !range_type)))
    return fail(ctx, PP_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  Cloud* c = nullptr;
  int rc = new_cloud(ctx, n, cloud, &c);
  if (rc) return rc;
  CK(ctx->gather_src.ensure(std::max<uint64_t>(n, 1) * 16));
  CK(cudaMemcpy(ctx->gather_src.p, pos_bytes, n * 16, cudaMemcpyHostToDevice));
  DevBuf rng;
  const size_t nr = (size_t)nranges;
  CK(rng.ensure(std::max<size_t>(nr, 1) * 9 + 64));
  float* dlo = rng.as<float>();
  float* dhi = dlo + std::max<size_t>(nr, 1);
  uint8_t* dty = (uint8_t*)(dhi + std::max<size_t>(nr, 1));
  if (nr) {
    CK(cudaMemcpy(dlo, range_lo, nr * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dhi, range_hi, nr * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dty, range_type, nr, cudaMemcpyHostToDevice));
  }
  pp::launch_decode_pos(ctx->gather_src.as<uint32_t>(), n, dlo, dhi, dty, nranges, c->xyz.as<float>(),
                        c->label.as<uint8_t>(), 0);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  return PP_OK;
}

int pp_cloud_free(pp_ctx* ctx, int cloud) {
  if (!ctx || !get_cloud(ctx, cloud)) return fail(ctx, PP_ERR_INVALID, "bad cloud");
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  // keep the buffers of up to kSpareClouds freed clouds for later uploads
  if (ctx->spare.size() < kSpareClouds) ctx->spare.push_back(std::move(ctx->clouds[cloud]));
  ctx->clouds[cloud].reset();
  if (ctx->geo_cloud == cloud) ctx->geo_cloud = -1;
  return PP_OK;
}

int pp_cloud_labels(pp_ctx* ctx, int cloud, uint8_t* out, uint64_t n) {
  Cloud* c = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!c || !out || n < c->n) return fail(ctx, PP_ERR_INVALID, "bad argument");
  CK(cudaMemcpy(out, c->label.p, c->n, cudaMemcpyDeviceToHost));
  return PP_OK;
}

int pp_hull_upload(pp_ctx* ctx, int cloud, const float* tri, uint64_t ntri, float carve_radius) {
  Cloud* c = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!c || (ntri && !tri) || !(carve_radius >= 0.f)) return fail(ctx, PP_ERR_INVALID, "bad argument");
  // one pass over the caller's vertices: all finite (else the cloud's hull is
  // left as it was), and their bounds
  float lo0 = INFINITY, lo1 = INFINITY, lo2 = INFINITY, hi0 = -INFINITY, hi1 = -INFINITY, hi2 = -INFINITY;
  bool finite = true;
  for (uint64_t i = 0; i < 3 * ntri; ++i) {
    const float x = tri[3 * i], y = tri[3 * i + 1], z = tri[3 * i + 2];
    finite &= std::isfinite(x) & std::isfinite(y) & std::isfinite(z);
    lo0 = std::fmin(lo0, x); hi0 = std::fmax(hi0, x);
    lo1 = std::fmin(lo1, y); hi1 = std::fmax(hi1, y);
    lo2 = std::fmin(lo2, z); hi2 = std::fmax(hi2, z);
  }
  if (!finite) return fail(ctx, PP_ERR_INVALID, "hull has non-finite vertices");
  c->hull.tri.assign(tri, tri + 9 * ntri);
  c->hull.lo[0] = lo0; c->hull.lo[1] = lo1; c->hull.lo[2] = lo2;
  c->hull.hi[0] = hi0; c->hull.hi[1] = hi1; c->hull.hi[2] = hi2;
  c->hull.carve = carve_radius;
  c->hull.present = ntri > 0;
  c->tri_ok = false;
  c->has_user_surf = false;
  c->surf_version = ~0ull;
  return PP_OK;
}

int pp_surfdist_upload(pp_ctx* ctx, int cloud, const float* d2) {
  Cloud* c = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!c || (c->n && !d2)) return fail(ctx, PP_ERR_INVALID, "bad argument");
  CK(c->user_surf.ensure(std::max<uint64_t>(c->n, 1) * 4));
  CK(cudaMemcpy(c->user_surf.p, d2, c->n * 4, cudaMemcpyHostToDevice));
  c->has_user_surf = true;
  c->surf_version = ~0ull;
  return PP_OK;
}

// NumberOfIonsInside / VolumeInside of the RDF header: the reference's
// occupancy grid (vxlizer::rectangular_binning and the steps it calls,
// src/PARAPROBE_SolverHdl.cpp:5059-5386).  The device bins every ion; the
// host labels the empty voxels in raster order with the Hoshen-Kopelman rules
// of src/PARAPROBE_HoshenKopelman.cpp:55-146 -- a voxel joins its labelled -x,
// -y and -z neighbours, except that with all three labelled only -y and -z are
// merged, and voxel 0 (label 0) stays unlabelled -- takes the cluster of the
// guard corner (0, 0, nz - 1) as vacuum (:5196-5270), marks the non-vacuum
// Moore neighbours of vacuum voxels off the border as surface (:5132-5194) and
// counts the rest as inside (:5059-5130).
int pp_cloud_inside(pp_ctx* ctx, int cloud, float bin_width_min, float bin_width_max, uint64_t* nions_inside,
                    float* volume_inside, uint64_t* voxels) {
  Cloud* cl = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!cl) return fail(ctx, PP_ERR_INVALID, "bad cloud");
  if (!(bin_width_min > 0.f) || !(bin_width_max > 0.f) || !std::isfinite(bin_width_min) || !std::isfinite(bin_width_max))
    return fail(ctx, PP_ERR_INVALID, "bin widths must be finite and positive");
  CK(cudaSetDevice(ctx->device));
  const uint64_t n = cl->n;
  cudaStream_t s = 0;
  // tip box (src/PARAPROBE_SolverHdl.cpp:1778-1791): min / max of every coordinate
  CK(ctx->bbox.ensure(8 * sizeof(uint32_t)));
  const uint32_t init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(ctx->bbox.p, init, sizeof init, cudaMemcpyHostToDevice, s));
  pp::launch_bbox(cl->xyz.as<float>(), n, ctx->bbox.as<float>(), s);
  uint32_t bb[8];
  CK(cudaMemcpyAsync(bb, ctx->bbox.p, sizeof bb, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (bb[6]) return fail(ctx, PP_ERR_INVALID, "cloud has %u non-finite coordinates", bb[6]);
  auto o2f = [](uint32_t o) {
    const uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
  };
  // define_vxlgrid (:5318-5340): box grown by one voxel, one more voxel each side
  const float w = (float)(0.5 * (double)(bin_width_min + bin_width_max));
  float lo[3];
  uint64_t nv[3];
  for (int k = 0; k < 3; ++k) {
    float a = n ? o2f(bb[k]) : std::numeric_limits<float>::max();
    float b = n ? o2f(bb[3 + k]) : std::numeric_limits<float>::lowest();
    a -= w;
    b += w;
    lo[k] = a;
    nv[k] = (uint64_t)std::ceil((b - a) / w) + 2;
  }
  const uint64_t nx = nv[0], ny = nv[1], nz = nv[2], nxy = nx * ny, nxyz = nxy * nz;
  if (nx >= 0xffffffffull || ny >= 0xffffffffull || nz >= 0xffffffffull || nxyz >= 0xffffffffull)
    return fail(ctx, PP_ERR_UNSUPPORTED, "the occupancy grid needs 2^32 or more voxels (the reference's limit too)");
  DevBuf occ_dev;
  CK(occ_dev.ensure(nxyz * 4));
  CK(cudaMemsetAsync(occ_dev.p, 0, nxyz * 4, s));
  CK(ctx->res.status.ensure(4));
  CK(cudaMemsetAsync(ctx->res.status.p, 0, 4, s));
  const uint32_t nv32[3] = {(uint32_t)nx, (uint32_t)ny, (uint32_t)nz};
  pp::launch_voxel_count(cl->xyz.as<float>(), n, lo, w, nv32, occ_dev.as<uint32_t>(), ctx->res.status.as<int>(), s);
  std::vector<uint32_t> occ(nxyz);
  int st = 0;
  CK(cudaMemcpyAsync(occ.data(), occ_dev.p, nxyz * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&st, ctx->res.status.p, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (st) return fail(ctx, PP_ERR_DEVICE, "an ion fell outside the occupancy grid");
  // Hoshen-Kopelman clusters of the empty voxels (union-find over voxel ids)
  std::vector<uint32_t> parent(nxyz);
  for (uint64_t b = 0; b < nxyz; ++b) parent[b] = (uint32_t)b;
  auto root = [&](uint32_t a) {
    while (parent[a] != a) {
      parent[a] = parent[parent[a]];
      a = parent[a];
    }
    return a;
  };
  auto join = [&](uint32_t a, uint32_t b) {
    a = root(a);
    b = root(b);
    if (a != b) parent[a] = b;
  };
  auto labelled = [&](uint64_t b) { return b != 0 && occ[b] == 0; };
  for (uint64_t z = 0; z < nz; ++z)
    for (uint64_t y = 0; y < ny; ++y)
      for (uint64_t x = 0; x < nx; ++x) {
        const uint64_t v = x + y * nx + z * nxy;
        if (!labelled(v)) continue;
        const bool lx = x > 0 && labelled(v - 1), ly = y > 0 && labelled(v - nx), lz = z > 0 && labelled(v - nxy);
        if (lx && ly && lz) {
          join((uint32_t)(v - nx), (uint32_t)(v - nxy));
          join((uint32_t)v, (uint32_t)(v - nx));
          continue;
        }
        if (lx) join((uint32_t)v, (uint32_t)(v - 1));
        if (ly) join((uint32_t)v, (uint32_t)(v - nx));
        if (lz) join((uint32_t)v, (uint32_t)(v - nxy));
      }
  std::vector<uint8_t> cls(nxyz, 0);  // 1 vacuum, 2 surface
  const uint64_t corner = (nz - 1) * nxy;
  if (labelled(corner)) {
    const uint32_t rc = root((uint32_t)corner);
    for (uint64_t b = 0; b < nxyz; ++b)
      if (labelled(b) && root((uint32_t)b) == rc) cls[b] = 1;
  }
  for (uint64_t z = 1; z + 1 < nz; ++z)
    for (uint64_t y = 1; y + 1 < ny; ++y)
      for (uint64_t x = 1; x + 1 < nx; ++x) {
        if (cls[x + y * nx + z * nxy] != 1) continue;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const uint64_t t = (x + dx) + (y + dy) * nx + (z + dz) * nxy;
              if ((dx || dy || dz) && cls[t] != 1) cls[t] = 2;
            }
      }
  uint64_t nvac = 0, nsrf = 0, nin = 0, ions_in = 0;
  for (uint64_t b = 0; b < nxyz; ++b) {
    if (cls[b] == 1) ++nvac;
    else if (cls[b] == 2) ++nsrf;
    else { ++nin; ions_in += occ[b]; }
  }
  float vol = (float)nin;
  vol *= w * w * w;
  if (nions_inside) *nions_inside = ions_in;
  if (volume_inside) *volume_inside = vol;
  if (voxels) {
    voxels[0] = nvac; voxels[1] = nsrf; voxels[2] = nin;
    voxels[3] = nx; voxels[4] = ny; voxels[5] = nz;
  }
  return PP_OK;
}

int pp_fetch_npcorr(pp_ctx* ctx, uint32_t* counts, uint64_t cap, uint64_t* edge) {
  if (!ctx || !ctx->res.valid || ctx->res.batched || !(ctx->res.plan.flags & PP_NPCORR))
    return fail(ctx, PP_ERR_STATE, "no pass with PP_NPCORR");
  const uint64_t e = ctx->res.plan.npc_edge;
  const uint64_t need = (uint64_t)ctx->res.ntasks * e * e * e;
  if (edge) *edge = e;
  if (!counts) return PP_OK;
  if (cap < need) return fail(ctx, PP_ERR_INVALID, "counts need %llu uint32", (unsigned long long)need);
  CK(cudaStreamSynchronize(ctx->res.stream));
  int st = 0;
  CK(cudaMemcpy(&st, ctx->res.status.p, 4, cudaMemcpyDeviceToHost));
  if (st) return fail(ctx, PP_ERR_DEVICE, "device status %d", st);
  CK(cudaMemcpy(counts, ctx->res.npc.p, need * 4, cudaMemcpyDeviceToHost));
  return PP_OK;
}

int pp_surfdist_fetch(pp_ctx* ctx, int cloud, float* out, uint64_t n) {
  Cloud* c = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!c || !out || n < c->n) return fail(ctx, PP_ERR_INVALID, "bad argument");
  if (!c->grid_ok || c->surf_version != c->grid_version) return fail(ctx, PP_ERR_STATE, "no ion2surf computed yet");
  CK(cudaDeviceSynchronize());
  std::vector<float> sorted(c->n);
  std::vector<uint32_t> slot(c->n);
  CK(cudaMemcpy(sorted.data(), c->surf.p, c->n * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(slot.data(), c->slot_of_id.p, c->n * 4, cudaMemcpyDeviceToHost));
  for (uint64_t i = 0; i < c->n; ++i) out[i] = sorted[slot[i]];
  return PP_OK;
}

int pp_tasks_set(pp_ctx* ctx, const uint32_t* trg_mask, const uint32_t* env_mask, int ntasks) {
  if (!ctx || ntasks < 0 || (ntasks && (!trg_mask || !env_mask))) return fail(ctx, PP_ERR_INVALID, "bad argument");
  ctx->trg.assign(trg_mask, trg_mask + 8 * (size_t)ntasks);
  ctx->env.assign(env_mask, env_mask + 8 * (size_t)ntasks);
  ctx->ntasks = ntasks;
  ctx->tasks_ok = true;
  ctx->geo_cloud = -1;
  return PP_OK;
}

int pp_hist_params(pp_ctx* ctx, float rmin, float rincr, float rmax) {
  if (!ctx) return PP_ERR_INVALID;
  if (!(rmax > 0.f) || !(rincr > 0.f) || !(rmin >= 0.f) || !(rmin < rmax) || !std::isfinite(rmax))
    return fail(ctx, PP_ERR_INVALID, "need 0 <= rmin < rmax and rincr > 0 (src/PARAPROBE_Settings.cpp:871-885)");
  set_tables(ctx->tab, rmin, rincr, rmax);
  ctx->hist_ok = true;
  return PP_OK;
}

}  // extern "C"

namespace {

// Stencil rows of a by x bz block of grid rows with sr rows on each side, as
// (ry, rz) offsets from (yb - sr, zb - sr), ordered by the squared gap (in
// cells) between the row and the block, then by rz and ry; cached per shape.
int ensure_block_rows(pp_ctx* ctx, int by, int bz, int sr, cudaStream_t s, const int16_t** out) {
  if (ctx->brows_key[0] != by || ctx->brows_key[1] != bz || ctx->brows_key[2] != sr) {
    const int ny = by + 2 * sr, nz = bz + 2 * sr;
    if (ny > 30000 || nz > 30000) return fail(ctx, PP_ERR_UNSUPPORTED, "cell block too large");
    auto gap = [sr](int r, int b) { return r < sr ? sr - r : (r >= sr + b ? r - (sr + b - 1) : 0); };
    std::vector<std::pair<int, int>> order;
    order.reserve((size_t)ny * nz);
    for (int rz = 0; rz < nz; ++rz)
      for (int ry = 0; ry < ny; ++ry) {
        const int gy = gap(ry, by), gz = gap(rz, bz);
        order.push_back({gy * gy + gz * gz, rz * ny + ry});
      }
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<int, int>& x, const std::pair<int, int>& y) { return x.first < y.first; });
    std::vector<int16_t> tab(order.size() * 2);
    for (size_t i = 0; i < order.size(); ++i) {
      tab[2 * i] = (int16_t)(order[i].second % ny);
      tab[2 * i + 1] = (int16_t)(order[i].second / ny);
    }
    CK(ctx->brows.ensure(tab.size() * 2));
    CK(cudaMemcpyAsync(ctx->brows.p, tab.data(), tab.size() * 2, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    ctx->brows_key[0] = by;
    ctx->brows_key[1] = bz;
    ctx->brows_key[2] = sr;
  }
  *out = ctx->brows.as<int16_t>();
  return PP_OK;
}

// Select the centres of a plain run into ctx->centres (cell order); returns
// their number.  Synchronises the stream once to learn the count.
int select_centres(pp_ctx* ctx, Cloud& cl, const uint8_t* labels, const float* surf, const int8_t* cslot, float R,
                   uint32_t* ncent, cudaStream_t s, const uint8_t* extra_slot_mask = nullptr) {
  const uint64_t n = cl.n;
  CK(ctx->centres.ensure(std::max<uint64_t>(n, 1) * 4));
  CK(ctx->centre_count.ensure(8));
  CK(ctx->sel_flags.ensure((n + 1) * 4));
  const uint64_t tmp_elems = (n + 1) / 2048 + 64;
  CK(ctx->sel_tmp.ensure(tmp_elems * 4 * 2));
  CK(ctx->cflag.ensure(std::max<uint64_t>(n, 1)));
  pp::launch_select_centres(labels ? labels : cl.label_sorted.as<uint8_t>(), surf, n, R * R, cslot,
                            extra_slot_mask, ctx->sel_flags.as<uint32_t>(), ctx->sel_tmp.as<uint32_t>(), tmp_elems * 2,
                            ctx->centres.as<uint32_t>(), ctx->centre_count.as<uint32_t>(), ctx->cflag.as<uint8_t>(), s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ncent, ctx->centre_count.p, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return PP_OK;
}

// One pass of compute_generic_spatstat3 on the device.  centre_limit > 0
// restricts the pass to the first centres (cell order), for tuning.
// labels_override (sorted-slot order) replaces the cloud's labels; no_miss
// drops the kNN miss dump (a centre without a neighbour adds nothing).
// centre_mask (host, input order, nullable): only ions with a nonzero byte
// may be centres, on top of the type and hull-distance filter.
int run_plain(pp_ctx* ctx, Cloud* cl, uint32_t flags, const uint32_t* k_list, int nk, const uint32_t* label_perm,
              cudaStream_t s, uint32_t centre_limit, const uint8_t* labels_override = nullptr,
              bool no_miss = false, const uint8_t* centre_mask = nullptr) {
  RunPlan P;
  int rc = make_plan(ctx, flags, k_list, nk, P);
  if (rc) return rc;
  const float R = ctx->tab.rmax;
  if ((rc = ensure_grid(ctx, *cl, R, s))) return rc;
  const float* surf = nullptr;
  if ((rc = ensure_surface(ctx, *cl, R, s, &surf))) return rc;
  const uint64_t n = cl->n;
  P.cmax = (flags & PP_CNTNB) ? 4095 : 0;  // neighbour counts above 4095 set PP_ERR_OVERFLOW
  DevTables D{};
  if ((rc = upload_tables(ctx, P, D, s))) return rc;
  if ((rc = alloc_result(ctx, P, 1, false, s))) return rc;
  // labels of this run
  const uint8_t* labels = nullptr;
  if (label_perm) {
    CK(ctx->perm_dev.ensure(std::max<uint64_t>(n, 1) * 4));
    CK(cudaMemcpyAsync(ctx->perm_dev.p, label_perm, n * 4, cudaMemcpyHostToDevice, s));
    CK(ctx->labels_run.ensure(std::max<uint64_t>(n, 1)));
    pp::launch_permute_labels(cl->label.as<uint8_t>(), ctx->perm_dev.as<uint32_t>(), cl->id_of_slot.as<uint32_t>(), n,
                              ctx->labels_run.as<uint8_t>(), s);
    labels = ctx->labels_run.as<uint8_t>();
  }
  if (labels_override) labels = labels_override;
  // caller's centre mask: input order -> sorted-slot order
  const uint8_t* mask_slot = nullptr;
  if (centre_mask) {
    CK(ctx->mask_in.ensure(std::max<uint64_t>(n, 1) * 2));
    uint8_t* m_in = ctx->mask_in.as<uint8_t>();
    CK(cudaMemcpyAsync(m_in, centre_mask, n, cudaMemcpyHostToDevice, s));
    pp::launch_gather_labels(m_in, cl->id_of_slot.as<uint32_t>(), n, m_in + n, 1, s);
    CK(cudaGetLastError());
    mask_slot = m_in + n;
  }
  uint32_t ncent = 0;
  if ((rc = select_centres(ctx, *cl, labels, surf, D.cslot, R, &ncent, s, mask_slot))) return rc;
  ctx->last_centres_all = ncent;
  // a tuning sample: every stride-th centre (or brick) over the whole cloud
  uint32_t stride = 1;
  if (centre_limit && ncent > centre_limit) {
    stride = ncent / centre_limit;
    ncent = ncent / stride;
  }
  ctx->res.ncentres_total = ncent;
  ctx->res.n_ions = n;
  // work counters of up to two launches, then pair / centre counters for a
  // second launch that must not count them again
  CK(ctx->work.ensure(32));
  CK(cudaMemsetAsync(ctx->work.p, 0, 32, s));
  pp::ScanArgs a{};
  fill_scan_common(a, *cl, P, D, ctx->tab);
  if (ctx->no_uniform) a.uniform_sets = 0;
  if (ctx->no_box) a.no_box_filter = 1;
  a.lists_mode = ctx->knn_lists;
  a.labels = labels;
  a.centres = ctx->centres.as<uint32_t>();
  a.ncentres = ncent;
  if (no_miss) a.cat_miss = -1;
  a.flags = flags & (PP_RDF | PP_RIPK | PP_CNTNB);
  if (flags & PP_RIPK) a.flags |= PP_RDF;
  a.rdf_core = ctx->res.rdf.as<unsigned long long>();
  a.knn_core = ctx->res.knn.as<unsigned long long>();
  a.cnt_core = ctx->res.cnt.as<unsigned long long>();
  a.cmax = P.cmax;
  a.counters = ctx->res.counters.as<unsigned long long>();
  CK(ctx->res.tests.ensure(8));
  CK(cudaMemsetAsync(ctx->res.tests.p, 0, 8, s));
  a.tests = ctx->res.tests.as<unsigned long long>();
  a.work = ctx->work.as<uint32_t>();
  a.status = ctx->res.status.as<int>();
  a.mode = 0;
  a.sample_stride = stride;
  a.rdf_in_smem = ((a.flags & PP_RDF) && (size_t)P.nC * P.nE * P.H * 4 <= 96 * 1024) ? 1 : 0;
  // a cell block set by tuning applies to every pass; one set by
  // pp_cloud_prepare only to passes of dense centres
  int dbx = 0, dby = 0, dbz = 0;
  const bool block_ok = cl->lanes_bx != 0 &&
                        (!cl->lanes_auto || default_block(*cl, (uint64_t)ncent * std::max<uint32_t>(stride, 1),
                                                          &dbx, &dby, &dbz));
  // RDF / RIPK and kNN in one pass on a cloud tuned to a centre-per-lane cell
  // block: two centre-per-lane passes, RDF / RIPK then kNN
  const bool split = P.kr > 0 && (a.flags & PP_RDF) && block_ok && !ctx->no_lanes &&
                     !(flags & (PP_CNTNB | PP_NPCORR));
  // RDF / RIPK alone: each pair of two centres is computed once and credited
  // to both (the counts are the same as the per-centre ball scan's)
  a.sym = ((P.kr == 0 || split) && !(flags & PP_CNTNB) && (a.flags & PP_RDF) && !ctx->no_sym) ? 1 : 0;
  a.cflag = ctx->cflag.as<uint8_t>();
  if (a.sym) {
    CK(ctx->nc_pre.ensure((cl->g.ncells + 1) * 4));
    const uint64_t tmp_elems = (cl->g.ncells + 1) / 2048 + 64;
    CK(ctx->scan_tmp.ensure(tmp_elems * 8 * 2));
    pp::launch_nc_prefix(cl->cell_start.as<uint32_t>(), cl->g.ncells, a.cflag, ctx->nc_pre.as<uint32_t>(),
                         ctx->scan_tmp.as<uint32_t>(), tmp_elems * 4, s);
    a.nc_pre = ctx->nc_pre.as<uint32_t>();
  }
  ctx->ev_recorded = false;
  if (ncent > 0) {
    size_t smem = 0;
    const Grid& g = cl->g;
    const bool rows_fit = (int)std::floor((R + 3.f * g.margin) * g.inv_h) + 1 <= 7;
    // centre-per-lane scans: cell block and its stencil rows
    bool lanes = rows_fit && !ctx->no_lanes && !(flags & (PP_CNTNB | PP_NPCORR)) &&
                 (split || !(P.kr > 0 && (a.flags & PP_RDF)));
    if (lanes && block_ok) {
      a.bx = (int)cl->lanes_bx;
      a.by = (int)std::max<uint32_t>(cl->lanes_by, 1);
      a.bz = (int)std::max<uint32_t>(cl->lanes_bz, 1);
    } else if (lanes) {
      lanes = default_block(*cl, (uint64_t)ncent * std::max<uint32_t>(stride, 1), &a.bx, &a.by, &a.bz);
    }
    a.bsr = (int)std::floor(((R + g.margin) + 2.f * g.margin) * g.inv_h) + 1;
    a.brows = nullptr;
    if (lanes && (rc = ensure_block_rows(ctx, a.by, a.bz, a.bsr, s, &a.brows)) != PP_OK) return rc;
    CK(cudaEventRecord(ctx->ev0, s));
    rc = -3;
    // passes with RDF / RIPK and kNN together take the per-centre scan, which
    // serves both from one candidate stream, unless the cloud is tuned to a
    // cell block (the autotuner times both): then the RDF / RIPK part and the
    // kNN part run as two centre-per-lane passes, the second on a fresh work
    // counter and with its pair and centre counts dropped (the first counted
    // them)
    if (rc == -3 && a.brows && split) {
      const uint64_t nb_x = ((uint64_t)g.nx + a.bx - 1) / a.bx, nb_y = ((uint64_t)g.ny + a.by - 1) / a.by;
      uint64_t nb = nb_x * nb_y * (((uint64_t)g.nz + a.bz - 1) / a.bz);
      if (stride > 1) nb = std::max<uint64_t>(1, nb / stride);
      if (nb < (1ull << 32)) {
        pp::ScanArgs ar = a;
        ar.nbricks = (uint32_t)nb;
        ar.tile = 4;
        rc = pp::launch_lanes(ar, 0, ctx->sm_count, &smem, s);
        if (rc == 0) {
          pp::ScanArgs ak = a;
          ak.flags &= ~(uint32_t)(PP_RDF | PP_RIPK);
          ak.sym = 0;
          ak.work = a.work + 1;
          ak.counters = (unsigned long long*)(ctx->work.as<unsigned char>() + 16);
          ak.nbricks = (uint32_t)nb;
          ak.tile = 4;
          rc = pp::launch_lanes_knn(ak, P.disjoint != 0, ctx->sm_count, &smem, s);
          ctx->last_kind = 4;
          if (rc == -3) {  // overlapping sets, or lists too large for shared memory
            ak.tile = a.tile;
            rc = pp::launch_scan(ak, P.kr, P.emax, ctx->sm_count, &smem, s);
            ctx->last_kind = 5;
          }
          if (rc == -3) rc = -1;  // the RDF part already ran
        }
      }
    }
    if (P.kr > 0) a.sym = 0;  // the per-centre scans need every centre's whole ball
    if (rc == -3 && a.brows && P.kr == 0 && (a.flags & PP_RDF)) {
      const uint64_t nb_x = ((uint64_t)g.nx + a.bx - 1) / a.bx, nb_y = ((uint64_t)g.ny + a.by - 1) / a.by;
      uint64_t nb = nb_x * nb_y * (((uint64_t)g.nz + a.bz - 1) / a.bz);
      if (stride > 1) nb = std::max<uint64_t>(1, nb / stride);
      if (nb < (1ull << 32)) {
        a.nbricks = (uint32_t)nb;
        const uint32_t keep = a.tile;
        a.tile = 4;  // bricks per warp work item
        rc = pp::launch_lanes(a, P.kr, ctx->sm_count, &smem, s);
        if (rc == 0) ctx->last_kind = 2;
        a.tile = keep;
      }
    }
    // kNN-only passes (with RDF in the same pass every in-ball pair would be
    // walked per lane; the per-centre scan does that pass better)
    if (rc == -3 && a.brows && P.kr > 0 && !(a.flags & PP_RDF)) {
      const uint64_t nb_x = ((uint64_t)g.nx + a.bx - 1) / a.bx, nb_y = ((uint64_t)g.ny + a.by - 1) / a.by;
      uint64_t nb = nb_x * nb_y * (((uint64_t)g.nz + a.bz - 1) / a.bz);
      if (stride > 1) nb = std::max<uint64_t>(1, nb / stride);
      if (nb < (1ull << 32)) {
        a.nbricks = (uint32_t)nb;
        const uint32_t keep = a.tile;
        a.tile = 4;  // blocks per warp work item
        rc = pp::launch_lanes_knn(a, P.disjoint != 0, ctx->sm_count, &smem, s);
        if (rc == 0) ctx->last_kind = 3;
        a.tile = keep;
      }
    }
    if (rc == -3 && cl->brick && rows_fit) {
      a.bx = (int)(cl->brick >> 16);
      a.bcap = (int)(cl->brick & 0xffffu);
      const uint64_t nbx = ((uint64_t)g.nx + a.bx - 1) / a.bx;
      uint64_t nb = nbx * g.ny * g.nz;
      if (stride > 1) nb = std::max<uint64_t>(1, nb / stride);
      if (nb < (1ull << 32)) {
        a.nbricks = (uint32_t)nb;
        const uint32_t keep = a.tile;
        a.tile = 16;
        rc = pp::launch_brick(a, P.kr, ctx->sm_count, &smem, s);
        if (rc == 0) ctx->last_kind = 1;
        a.tile = keep;
      }
    }
    if (rc == -3) {
      rc = pp::launch_scan(a, P.kr, P.emax, ctx->sm_count, &smem, s);
      ctx->last_kind = 0;
    }
    if (rc == 0 && (flags & PP_NPCORR)) {
      pp::NpcArgs np{};
      np.id_of_slot = cl->id_of_slot.as<uint32_t>();
      np.K = P.npc_K;
      np.ntk = D.ntk;
      np.tk_task = D.tk_task;
      np.tk_set = D.tk_set;
      np.half = P.npc_half;
      np.edge = P.npc_edge;
      np.inv_w = 1.f / ctx->tab.rincr;
      np.rmax = ctx->tab.rmax;
      np.counts = ctx->res.npc.as<uint32_t>();
      pp::ScanArgs an = a;
      an.sample_stride = 0;
      an.sym = 0;  // every centre needs its whole ball, not the pairs it owns
      rc = pp::launch_npcorr(an, np, ctx->sm_count, s);
      if (rc) {
        CK(cudaEventRecord(ctx->ev1, s));
        ctx->ev_recorded = true;
        return fail(ctx, PP_ERR_CUDA, "n-point correlation launch failed");
      }
    }
    CK(cudaEventRecord(ctx->ev1, s));
    ctx->ev_recorded = true;
    if (rc == -2) return fail(ctx, PP_ERR_UNSUPPORTED, "no kernel variant for k=%d with %d environment sets", P.kmax, P.emax);
    if (rc) {
      cudaError_t e = cudaGetLastError();
      return fail(ctx, PP_ERR_CUDA, "scan launch failed (%s, %zu B shared)", cudaGetErrorString(e), smem);
    }
  }
  ctx->res.valid = true;
  ctx->res.centres_sel.assign(1, ncent);
  return PP_OK;
}

}  // namespace

extern "C" {

int pp_run(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk, const uint32_t* label_perm,
           void* stream) {
  if (!ctx) return PP_ERR_INVALID;
  Cloud* cl = get_cloud(ctx, cloud);
  if (!cl) return fail(ctx, PP_ERR_INVALID, "bad cloud");
  CK(cudaSetDevice(ctx->device));
  return run_plain(ctx, cl, flags, k_list, nk, label_perm, (cudaStream_t)stream, 0);
}

int pp_run_masked(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk, const uint32_t* label_perm,
                  const uint8_t* centre_mask, void* stream) {
  if (!ctx) return PP_ERR_INVALID;
  Cloud* cl = get_cloud(ctx, cloud);
  if (!cl) return fail(ctx, PP_ERR_INVALID, "bad cloud");
  if (!centre_mask) return fail(ctx, PP_ERR_INVALID, "centre_mask is NULL (use pp_run)");
  CK(cudaSetDevice(ctx->device));
  return run_plain(ctx, cl, flags, k_list, nk, label_perm, (cudaStream_t)stream, 0, nullptr, false, centre_mask);
}

// Statistics after clustering (clustertask::flag2exclude_guard and
// generic_spatstat, src/PARAPROBE_SolverHdl.cpp:4790-4945).  The device labels
// of this pass are 1 (neither clustered nor guard: centre and environment),
// 2 (guard: environment only) and 3 (clustered: neither); one internal task
// takes label 1 as targets and labels 1 and 2 as environment, so the plain
// pass computes exactly the reference's per-centre loop.  The caller's tasks
// are put back afterwards.
int pp_run_aposteriori(pp_ctx* ctx, int cloud, const uint8_t* clustered, uint32_t flags, void* stream) {
  if (!ctx) return PP_ERR_INVALID;
  Cloud* cl = get_cloud(ctx, cloud);
  if (!cl || !clustered) return fail(ctx, PP_ERR_INVALID, "bad argument");
  if (!flags || (flags & ~(uint32_t)(PP_RDF | PP_1NN | PP_RIPK)))
    return fail(ctx, PP_ERR_INVALID, "flags: a combination of PP_RDF, PP_1NN and PP_RIPK");
  if (!ctx->hist_ok) return fail(ctx, PP_ERR_STATE, "pp_hist_params was not called");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t n = cl->n;
  const std::vector<uint32_t> keep_trg = ctx->trg, keep_env = ctx->env;
  const int keep_nt = ctx->ntasks;
  const bool keep_ok = ctx->tasks_ok;
  ctx->trg.assign(8, 0u);
  ctx->env.assign(8, 0u);
  ctx->trg[0] = 1u << 1;
  ctx->env[0] = (1u << 1) | (1u << 2);
  ctx->ntasks = 1;
  ctx->tasks_ok = true;
  int rc = PP_OK;
  do {
    RunPlan P;
    if ((rc = make_plan(ctx, flags, nullptr, 0, P))) break;
    if ((rc = ensure_grid(ctx, *cl, ctx->tab.rmax, s))) break;
    DevTables D{};
    if ((rc = upload_tables(ctx, P, D, s))) break;
    // [clustered flags by slot | guard flags, then labels | status word]
    const uint64_t stat_off = (2 * n + 15) & ~uint64_t(15);
    if (ctx->gather_src.ensure(std::max<uint64_t>(n, 1)) != cudaSuccess ||
        ctx->perm_dev.ensure(stat_off + 16) != cudaSuccess) {
      rc = fail(ctx, PP_ERR_NOMEM, "device allocation failed");
      break;
    }
    uint8_t* clus = ctx->perm_dev.as<uint8_t>();
    uint8_t* lab = clus + n;
    int* gstat = reinterpret_cast<int*>(clus + stat_off);
    if (cudaMemcpyAsync(ctx->gather_src.p, clustered, n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(lab, 0, n, s) != cudaSuccess || cudaMemsetAsync(gstat, 0, 4, s) != cudaSuccess) {
      rc = fail(ctx, PP_ERR_CUDA, "copy of the cluster flags failed");
      break;
    }
    pp::ScanArgs a{};
    fill_scan_common(a, *cl, P, D, ctx->tab);
    a.status = gstat;
    if (ctx->apost_ref) {
      // The guard loop as the reference runs it (src/PARAPROBE_SolverHdl.cpp:4804-4820):
      // for every position i of ions_kdtree in order whose ion is clustered,
      // it relabels the ions at positions 0 .. |ball(i)| - 1 -- the loop
      // reads ions_kdtree.at(cand), cand being the index into the result
      // list -- with i's clustered type (flag_as_guarded returns a clustered
      // type unchanged, :4576-4582), so they are clustered from then on and
      // later steps take them as clustered ions too.  Positions are the
      // cloud's input order.  The relabelled ions form the prefix [0, G) of
      // positions, G the largest ball of a clustered position met while the
      // prefix is extended; they leave the statistics as centres and as
      // neighbours (:4879, :4890, :4898).
      if (ctx->apost_cnt.ensure(std::max<uint64_t>(n, 1) * 4) != cudaSuccess) {
        rc = fail(ctx, PP_ERR_NOMEM, "device allocation failed");
        break;
      }
      pp::launch_ball_count(a, cl->id_of_slot.as<uint32_t>(), n, ctx->apost_cnt.as<uint32_t>(), ctx->sm_count, s);
      std::vector<uint32_t> ball(n);
      int st = 0;
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(ball.data(), ctx->apost_cnt.p, n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaMemcpyAsync(&st, gstat, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) {
        rc = fail(ctx, PP_ERR_CUDA, "neighbour count pass failed");
        break;
      }
      if (st) {
        rc = fail(ctx, PP_ERR_DEVICE, "neighbour count pass: device status %d", st);
        break;
      }
      uint64_t G = 0;
      for (uint64_t i = 0; i < n; ++i)
        if (clustered[i] || i < G) G = std::max<uint64_t>(G, ball[i]);
      std::vector<uint8_t> lab_in(n);
      uint64_t relabelled = 0;
      for (uint64_t i = 0; i < n; ++i) {
        const bool out = clustered[i] || i < G;
        lab_in[i] = out ? 3 : 1;
        relabelled += (!clustered[i] && i < G) ? 1 : 0;
      }
      ctx->apost_relabelled = relabelled;
      if (cudaMemcpyAsync(ctx->gather_src.p, lab_in.data(), n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
        rc = fail(ctx, PP_ERR_CUDA, "copy of the labels failed");
        break;
      }
      pp::launch_gather_labels(ctx->gather_src.as<uint8_t>(), cl->id_of_slot.as<uint32_t>(), n, lab, 1, s);
      if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
        rc = fail(ctx, PP_ERR_CUDA, "label gather failed");
        break;
      }
      rc = run_plain(ctx, cl, flags, nullptr, 0, nullptr, s, 0, lab, true);
      break;
    }
    pp::launch_gather_labels(ctx->gather_src.as<uint8_t>(), cl->id_of_slot.as<uint32_t>(), n, clus, 1, s);
    pp::launch_guard(a, clus, lab, n, ctx->sm_count, s);
    int st = 0;
    if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&st, gstat, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      rc = fail(ctx, PP_ERR_CUDA, "guard zone pass failed");
      break;
    }
    if (st) {
      rc = fail(ctx, PP_ERR_DEVICE, "guard zone pass: device status %d", st);
      break;
    }
    rc = run_plain(ctx, cl, flags, nullptr, 0, nullptr, s, 0, lab, true);
  } while (false);
  ctx->trg = keep_trg;
  ctx->env = keep_env;
  ctx->ntasks = keep_nt;
  ctx->tasks_ok = keep_ok;
  ctx->geo_cloud = -1;
  return rc;
}

// Times the scan on the first `sample` centres for each candidate cell ratio
// (R / h) and block tile, keeps the fastest pair for this cloud and rebuilds
// its grid.  Uses the current tasks and histogram settings.
int pp_autotune(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk, uint32_t sample,
                float* best_ratio, uint32_t* best_tile) {
  if (!ctx) return PP_ERR_INVALID;
  Cloud* cl = get_cloud(ctx, cloud);
  if (!cl) return fail(ctx, PP_ERR_INVALID, "bad cloud");
  CK(cudaSetDevice(ctx->device));
  if (sample == 0) sample = 200000;
  // The sample must fill the GPU several times over, or kernels whose work
  // items hold many centres (the centre-per-lane scans: a warp takes four cell
  // blocks of about a warp of centres at once) run partly idle and rank below
  // the per-centre scan although they win on the whole cloud: at least 8192
  // centres per SM (four work items for each of 64 warps).
  sample = std::max<uint32_t>(sample, (uint32_t)ctx->sm_count * 8192u);
  const float R = ctx->tab.rmax;
  const float ratios[] = {2.0f, 3.0f, 4.0f, 5.0f};
  auto lanes_code = [](uint32_t bx, uint32_t by, uint32_t bz) {
    return ((bx | by << 8 | bz << 12) << 16) | PP_TILE_LANES;
  };
  // passes the centre-per-lane scan takes: cell blocks of about 2 x 1 x 1 R/2
  // (a few tens of centres at atom-probe densities) for each cell edge
  const uint32_t lanes_tiles[4][2] = {{lanes_code(2, 1, 1), lanes_code(2, 2, 1)},
                                      {lanes_code(3, 2, 2), lanes_code(2, 2, 2)},
                                      {lanes_code(4, 2, 2), lanes_code(4, 3, 3)},
                                      {lanes_code(5, 3, 3), lanes_code(4, 4, 4)}};
  // other passes: per-centre tiles, then brick codes (cells per brick << 16 | batch)
  const uint32_t scan_tiles[] = {32, 128, 512, (4u << 16) | 16u, (8u << 16) | 16u, (8u << 16) | 32u,
                                 (16u << 16) | 32u};
  const float keep_ratio = cl->cell_ratio;
  const uint32_t keep[5] = {cl->tile, cl->brick, cl->lanes_bx, cl->lanes_by, cl->lanes_bz};
  const bool keep_auto = cl->lanes_auto;
  cl->lanes_auto = false;  // the trials' cell blocks apply as tuned
  auto apply = [&](uint32_t t) {
    if (t >= 65536u && (t & 0xffffu) == PP_TILE_LANES) {
      cl->lanes_bx = (t >> 16) & 0xffu;
      cl->lanes_by = (t >> 24) & 0xfu;
      cl->lanes_bz = t >> 28;
    } else if (t >= 65536u) {
      cl->brick = t;
      cl->lanes_bx = cl->lanes_by = cl->lanes_bz = 0;
    } else {
      cl->tile = t;
      cl->brick = 0;
      cl->lanes_bx = cl->lanes_by = cl->lanes_bz = 0;
    }
  };
  // RDF / RIPK with kNN in one pass: the per-centre scan's tiles and the two
  // centre-per-lane passes a cell block gives
  const bool combined = (flags & (PP_RDF | PP_RIPK)) && (flags & (PP_1NN | PP_MKNN)) &&
                        !(flags & (PP_CNTNB | PP_NPCORR)) && !ctx->no_lanes;
  float bestr = keep_ratio, bestms = 1e30f;
  uint32_t bestt = 0;
  int rc = PP_OK;
  for (int ri = 0; ri < 4 && rc == PP_OK; ++ri) {
    cl->cell_ratio = ratios[ri];
    if ((rc = build_grid(ctx, *cl, R, 0))) break;
    // which kernel does this pass take at this cell edge?
    cl->lanes_bx = cl->lanes_by = cl->lanes_bz = 0;
    if ((rc = run_plain(ctx, cl, flags, k_list, nk, nullptr, 0, sample))) break;
    const bool lanes = ctx->last_kind >= 2;
    // two fixed cell-block shapes; for RDF / RIPK with kNN also the default
    // block at this cell edge (about a warp of centres), as the fixed shapes
    // are sized for R = 2 nm at atom-probe densities.  (Offered to single
    // passes too, the default block won on the tuning sample but lost on the
    // whole 20M-ion tip, so they keep the two shapes.)
    int dbx = 0, dby = 0, dbz = 0;
    const bool dense = combined && default_block(*cl, ctx->last_centres_all, &dbx, &dby, &dbz);
    uint32_t tiles[sizeof scan_tiles / sizeof scan_tiles[0] + 3];
    int ntiles = 0;
    if (!lanes)
      for (uint32_t t : scan_tiles) tiles[ntiles++] = t;
    if (lanes || dense) {
      const uint32_t dcode = (!lanes && dense) ? lanes_code((uint32_t)dbx, (uint32_t)dby, (uint32_t)dbz) : 0u;
      if (dcode && dcode != lanes_tiles[ri][0] && dcode != lanes_tiles[ri][1]) tiles[ntiles++] = dcode;
      tiles[ntiles++] = lanes_tiles[ri][0];
      tiles[ntiles++] = lanes_tiles[ri][1];
    }
    for (int ti = 0; ti < ntiles && rc == PP_OK; ++ti) {
      apply(tiles[ti]);
      float ms = 0.f;
      for (int rep = 0; rep < 2 && rc == PP_OK; ++rep) {  // first repetition warms caches and lazy state
        if ((rc = run_plain(ctx, cl, flags, k_list, nk, nullptr, 0, sample))) break;
        rc = pp_last_kernel_ms(ctx, &ms);
      }
      if (rc == PP_OK && ms < bestms) { bestms = ms; bestr = ratios[ri]; bestt = tiles[ti]; }
    }
    cl->tile = keep[0];
    cl->brick = keep[1];
    cl->lanes_bx = keep[2];
    cl->lanes_by = keep[3];
    cl->lanes_bz = keep[4];
  }
  if (rc != PP_OK) {
    cl->cell_ratio = keep_ratio;
    cl->lanes_auto = keep_auto;
    build_grid(ctx, *cl, R, 0);
    return rc;
  }
  cl->cell_ratio = bestr;
  if (bestt) apply(bestt);
  else cl->lanes_auto = keep_auto;
  if ((rc = build_grid(ctx, *cl, R, 0))) return rc;
  ctx->res.valid = false;
  if (best_ratio) *best_ratio = bestr;
  if (best_tile) *best_tile = bestt;
  return PP_OK;
}

int pp_fp64_audit(pp_ctx* ctx, int cloud, uint32_t max_centres, double* max_abs, double* max_rel, uint64_t* pairs,
                  uint64_t* bin_disagree, uint64_t* set_disagree, uint64_t* listing_ids, double* listing_d,
                  uint64_t cap, uint64_t* nlisted) {
  if (!ctx) return PP_ERR_INVALID;
  Cloud* cl = get_cloud(ctx, cloud);
  if (!cl) return fail(ctx, PP_ERR_INVALID, "bad cloud");
  if (cap && (!listing_ids || !listing_d)) return fail(ctx, PP_ERR_INVALID, "listing buffers missing");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = 0;
  RunPlan P;
  int rc = make_plan(ctx, PP_RDF, nullptr, 0, P);
  if (rc) return rc;
  const float R = ctx->tab.rmax;
  if ((rc = ensure_grid(ctx, *cl, R, s))) return rc;
  const float* surf = nullptr;
  if ((rc = ensure_surface(ctx, *cl, R, s, &surf))) return rc;
  DevTables D{};
  if ((rc = upload_tables(ctx, P, D, s))) return rc;
  uint32_t ncent = 0;
  if ((rc = select_centres(ctx, *cl, nullptr, surf, D.cslot, R, &ncent, s))) return rc;
  const uint32_t take = (max_centres && max_centres < ncent) ? max_centres : ncent;
  const uint32_t stride = take ? std::max<uint32_t>(1, ncent / std::max<uint32_t>(take, 1)) : 1;
  pp::ScanArgs a{};
  fill_scan_common(a, *cl, P, D, ctx->tab);
  const float Rw = R * (1.0f + 1.0f / 1024.0f);  // candidates slightly beyond R (double may include them)
  a.R = Rw;
  a.Rm2 = (Rw + cl->g.margin) * (Rw + cl->g.margin);
  a.centres = ctx->centres.as<uint32_t>();
  a.ncentres = take;
  a.status = nullptr;
  a.sym = 0;
  DevBuf out, ls, ld;
  const uint64_t c = std::min<uint64_t>(cap, 1u << 20);
  CK(out.ensure(8 * 8));
  CK(cudaMemset(out.p, 0, 8 * 8));
  CK(ls.ensure(std::max<uint64_t>(c, 1) * 8));
  CK(ld.ensure(std::max<uint64_t>(c, 1) * 16));
  int* status = nullptr;
  CK(cudaMalloc(&status, 4));
  CK(cudaMemset(status, 0, 4));
  a.status = status;
  pp::launch_audit(a, ctx->tab.hstart, ctx->tab.hscale, ctx->tab.hend, (double)R, (int)ctx->tab.nbins, stride,
                   out.as<unsigned long long>(), ls.as<uint32_t>(), ld.as<double>(), (uint32_t)c, ctx->sm_count, s);
  unsigned long long o[8];
  const cudaError_t e = cudaMemcpy(o, out.p, sizeof o, cudaMemcpyDeviceToHost);
  cudaFree(status);
  CK(e);
  double v;
  std::memcpy(&v, &o[0], 8);
  if (max_abs) *max_abs = v;
  std::memcpy(&v, &o[1], 8);
  if (max_rel) *max_rel = v;
  if (pairs) *pairs = o[2];
  if (bin_disagree) *bin_disagree = o[3];
  if (set_disagree) *set_disagree = o[4];
  const uint64_t nl = std::min<uint64_t>(o[5], c);
  if (nlisted) *nlisted = nl;
  if (nl) {
    std::vector<uint32_t> slots(2 * nl), id_of(cl->n);
    std::vector<double> dd(2 * nl);
    CK(cudaMemcpy(slots.data(), ls.p, nl * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dd.data(), ld.p, nl * 16, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(id_of.data(), cl->id_of_slot.p, cl->n * 4, cudaMemcpyDeviceToHost));
    for (uint64_t k = 0; k < nl; ++k) {
      for (int j = 0; j < 2; ++j) {
        const uint32_t idx = id_of[slots[2 * k + j]];
        listing_ids[2 * k + j] = cl->ids.empty() ? (uint64_t)idx : (uint64_t)cl->ids[idx];
        listing_d[2 * k + j] = dd[2 * k + j];
      }
    }
  }
  return PP_OK;
}

int pp_set_option(pp_ctx* ctx, const char* name, int value) {
  if (!ctx || !name) return PP_ERR_INVALID;
  if (std::strcmp(name, "symmetric") == 0) { ctx->no_sym = (value == 0); return PP_OK; }
  if (std::strcmp(name, "lanes") == 0) { ctx->no_lanes = (value == 0); return PP_OK; }
  if (std::strcmp(name, "uniform_sets") == 0) { ctx->no_uniform = (value == 0); return PP_OK; }
  if (std::strcmp(name, "box_filter") == 0) { ctx->no_box = (value == 0); return PP_OK; }
  if (std::strcmp(name, "knn_lists") == 0) {
    if (value < 0 || value > 2) return fail(ctx, PP_ERR_INVALID, "knn_lists must be 0, 1 or 2");
    ctx->knn_lists = value;
    return PP_OK;
  }
  if (std::strcmp(name, "npcorr_order") == 0) {
    if (value < 0 || value > 31) return fail(ctx, PP_ERR_INVALID, "npcorr_order must be in [0, 31]");
    ctx->npc_order = (uint32_t)value;
    return PP_OK;
  }
  if (std::strcmp(name, "server_batch") == 0) {
    if (value < 1 || value > pp::kMultiMaxQueries)
      return fail(ctx, PP_ERR_INVALID, "server_batch must be in [1, %d]", pp::kMultiMaxQueries);
    ctx->server_batch = value;
    return PP_OK;
  }
  if (std::strcmp(name, "aposteriori_guard") == 0) {
    if (value < 0 || value > 1) return fail(ctx, PP_ERR_INVALID, "aposteriori_guard must be 0 or 1");
    ctx->apost_ref = value == 1;
    return PP_OK;
  }
  if (std::strcmp(name, "batched_pair_cap") == 0) {
    if (value < 0) return fail(ctx, PP_ERR_INVALID, "batched_pair_cap must be >= 0");
    ctx->pair_cap_opt = (uint64_t)value;
    return PP_OK;
  }
  return fail(ctx, PP_ERR_INVALID, "unknown option %s", name);
}

int pp_cloud_tuning(pp_ctx* ctx, int cloud, float cell_ratio, uint32_t tile) {
  Cloud* cl = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!cl || !(cell_ratio >= 1.0f && cell_ratio <= 8.0f) || tile == 0)
    return fail(ctx, PP_ERR_INVALID, "cell_ratio in [1, 8] and a tile code required");
  if (tile >= 65536u && (tile & 0xffffu) == PP_TILE_LANES) {
    const uint32_t bx = (tile >> 16) & 0xffu, by = (tile >> 24) & 0xfu, bz = tile >> 28;
    if (bx < 1 || bx > 64)
      return fail(ctx, PP_ERR_INVALID, "centre-per-lane code: (bx | by << 8 | bz << 12) << 16, bx in [1, 64]");
    cl->lanes_bx = bx;
    cl->lanes_by = by ? by : 1;
    cl->lanes_bz = bz ? bz : 1;
    cl->lanes_auto = false;
  } else if (tile >= 65536u) {
    const uint32_t bx = tile >> 16, cap = tile & 0xffffu;
    if (bx < 1 || bx > 64 || cap < 1 || cap > 32)
      return fail(ctx, PP_ERR_INVALID, "brick code: cells per brick in [1, 64] << 16 | batch in [1, 32]");
    cl->brick = tile;
  } else {
    cl->tile = tile;
    cl->brick = 0;
  }
  if (cl->cell_ratio != cell_ratio) cl->grid_ok = false;
  cl->cell_ratio = cell_ratio;
  return PP_OK;
}

int pp_result_size(pp_ctx* ctx, uint64_t* total, uint64_t* nbins) {
  if (!ctx || !ctx->res.valid) return fail(ctx, PP_ERR_STATE, "no run");
  if (total) *total = result_len(ctx->res);
  if (nbins) *nbins = ctx->res.nbins;
  return PP_OK;
}

int pp_fetch(pp_ctx* ctx, uint64_t* bins, size_t cap) {
  if (!ctx) return PP_ERR_INVALID;
  int rc = fetch_cores(ctx);
  if (rc) return rc;
  const uint64_t need = result_len(ctx->res);
  if (!bins || cap < need) return fail(ctx, PP_ERR_INVALID, "result needs %llu uint64", (unsigned long long)need);
  finalize(ctx->res, 0, bins);
  return PP_OK;
}

int pp_fetch_cntnb(pp_ctx* ctx, uint64_t* bins, size_t cap, uint64_t* len) {
  if (!ctx || !len) return PP_ERR_INVALID;
  int rc = fetch_cores(ctx);
  if (rc) return rc;
  const Result& R = ctx->res;
  const RunPlan& P = R.plan;
  if (!(P.flags & PP_CNTNB) || R.batched) return fail(ctx, PP_ERR_STATE, "last run had no PP_CNTNB");
  const int W = P.cmax + 1;
  // common length: largest nonzero count + 1 over all tasks
  uint64_t L = 0;
  std::vector<std::vector<unsigned long long>> per(R.ntasks, std::vector<unsigned long long>(W, 0));
  for (int t = 0; t < R.ntasks; ++t) {
    for (int c = 0; c < P.nC; ++c) {
      if (!has_type(&R.trg[8 * t], P.ctype[c])) continue;
      for (int e = 0; e < P.nE; ++e) {
        if (!has_type(&R.env[8 * t], P.etype[e])) continue;
        const unsigned long long* src = R.cnt_h.data() + ((size_t)c * P.nE + e) * W;
        for (int v = 0; v < W; ++v) per[t][v] += src[v];
      }
    }
    for (int v = W - 1; v >= 0; --v)
      if (per[t][v]) { L = std::max<uint64_t>(L, (uint64_t)v + 1); break; }
  }
  *len = L;
  if (!bins) return PP_OK;
  if (cap < L * (uint64_t)R.ntasks) return fail(ctx, PP_ERR_INVALID, "cntnb needs %llu uint64", (unsigned long long)(L * R.ntasks));
  for (int t = 0; t < R.ntasks; ++t)
    for (uint64_t v = 0; v < L; ++v) bins[(uint64_t)t * L + v] = per[t][v];
  return PP_OK;
}

int pp_run_stats(pp_ctx* ctx, uint64_t* centres, uint64_t* discarded, uint64_t* pairs) {
  if (!ctx) return PP_ERR_INVALID;
  int rc = fetch_cores(ctx);
  if (rc) return rc;
  const Result& R = ctx->res;
  if (centres) *centres = R.counters_h[1];
  if (discarded) *discarded = R.n_ions - R.counters_h[1];
  if (pairs) *pairs = R.counters_h[0];
  return PP_OK;
}

int pp_neighbors(pp_ctx* ctx, int cloud, uint64_t ion, float r, uint64_t* ids, float* d2, uint64_t cap,
                 uint64_t* count) {
  Cloud* cl = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!cl || ion >= cl->n || !count || !(r > 0.f)) return fail(ctx, PP_ERR_INVALID, "bad argument");
  CK(cudaSetDevice(ctx->device));
  int rc = ensure_grid(ctx, *cl, r, 0);
  if (rc) return rc;
  uint32_t self = 0;
  CK(cudaMemcpy(&self, cl->slot_of_id.as<uint32_t>() + ion, 4, cudaMemcpyDeviceToHost));
  const uint32_t dcap = 1u << 22;
  DevBuf bs, bd, bc;
  CK(bs.ensure(dcap * 4));
  CK(bd.ensure(dcap * 4));
  CK(bc.ensure(4));
  CK(cudaMemset(bc.p, 0, 4));
  pp::launch_neighbors(cl->ions.as<float4>(), cl->cell_start.as<uint32_t>(), cl->g, self, r, nullptr,
                       bs.as<uint32_t>(), bd.as<float>(), dcap, bc.as<uint32_t>(), 0);
  CK(cudaGetLastError());
  uint32_t cnt = 0;
  CK(cudaMemcpy(&cnt, bc.p, 4, cudaMemcpyDeviceToHost));
  if (cnt > dcap) return fail(ctx, PP_ERR_OVERFLOW, "more than %u neighbours", dcap);
  std::vector<uint32_t> slots(cnt), id_of(cl->n);
  std::vector<float> dd(cnt);
  CK(cudaMemcpy(slots.data(), bs.p, cnt * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(dd.data(), bd.p, cnt * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(id_of.data(), cl->id_of_slot.p, cl->n * 4, cudaMemcpyDeviceToHost));
  std::vector<std::pair<float, uint64_t>> v(cnt);
  for (uint32_t k = 0; k < cnt; ++k) {
    const uint32_t idx = id_of[slots[k]];
    v[k] = {dd[k], cl->ids.empty() ? (uint64_t)idx : (uint64_t)cl->ids[idx]};
  }
  std::sort(v.begin(), v.end());
  *count = cnt;
  for (uint64_t k = 0; k < cnt && k < cap; ++k) {
    if (ids) ids[k] = v[k].second;
    if (d2) d2[k] = v[k].first;
  }
  return PP_OK;
}

int pp_shuffle_labels(const uint8_t* label, uint64_t n, uint64_t seed, uint8_t* out) {
  if ((n && (!label || !out))) return PP_ERR_INVALID;
  pp_host::shuffle_labels(label, n, seed, out);
  return PP_OK;
}

// ------------------------------------------------------------- batched
int pp_run_batched(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk, int include_original,
                   const uint8_t* label_sets, int n_label_sets, const float* rois, int n_rois, void* stream) {
  if (!ctx) return PP_ERR_INVALID;
  Cloud* cl = get_cloud(ctx, cloud);
  if (!cl) return fail(ctx, PP_ERR_INVALID, "bad cloud");
  if (n_label_sets < 0 || n_rois < 0 || (n_label_sets && !label_sets) || (n_rois && !rois))
    return fail(ctx, PP_ERR_INVALID, "bad realisation arguments");
  if (flags & (PP_CNTNB | PP_NPCORR)) return fail(ctx, PP_ERR_UNSUPPORTED, "PP_CNTNB and PP_NPCORR are provided by pp_run only");
  const int nreal = (include_original ? 1 : 0) + n_label_sets + n_rois;
  if (nreal == 0) return fail(ctx, PP_ERR_INVALID, "no realisation requested");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  RunPlan P;
  int rc = make_plan(ctx, flags, k_list, nk, P);
  if (rc) return rc;
  if (P.H > 65535) return fail(ctx, PP_ERR_UNSUPPORTED, "batched runs hold categories in 16 bits");
  const float R = ctx->tab.rmax;
  if ((rc = ensure_grid(ctx, *cl, R, s))) return rc;
  const float* surf = nullptr;
  if ((rc = ensure_surface(ctx, *cl, R, s, &surf))) return rc;
  const uint64_t n = cl->n;
  DevTables D{};
  if ((rc = upload_tables(ctx, P, D, s))) return rc;
  if ((rc = alloc_result(ctx, P, nreal, true, s))) return rc;

  // ---- geometry: per-centre pair lists sorted by category (cached)
  const bool geo_hit = ctx->geo_cloud == cloud && ctx->geo_key_version == cl->grid_version && ctx->geo_R == R &&
                       ctx->geo_H == P.H && ctx->geo_rmin == ctx->tab.rmin && ctx->geo_rincr == ctx->tab.rincr &&
                       cl->surf_version == cl->grid_version;
  ctx->ev_recorded = false;
  if (!geo_hit) {
    uint32_t nc = 0;
    if ((rc = select_centres(ctx, *cl, nullptr, surf, nullptr, R, &nc, s))) return rc;
    CK(ctx->geo_centres.ensure(std::max<uint64_t>(n, 1) * 4));
    CK(cudaMemcpyAsync(ctx->geo_centres.p, ctx->centres.p, (uint64_t)nc * 4, cudaMemcpyDeviceToDevice, s));
    pp::ScanArgs a{};
    fill_scan_common(a, *cl, P, D, ctx->tab);
    a.labels = cl->label_sorted.as<uint8_t>();
    a.centres = ctx->geo_centres.as<uint32_t>();
    a.ncentres = nc;
    a.flags = 0;
    CK(ctx->geo_counters.ensure(16));
    a.counters = ctx->geo_counters.as<unsigned long long>();
    a.status = ctx->res.status.as<int>();
    a.rdf_in_smem = 0;
    CK(ctx->work.ensure(16));
    CK(ctx->pair_count.ensure((std::max<uint64_t>(nc, 1)) * 4));
    CK(ctx->pair_off.ensure((std::max<uint64_t>(nc, 1) + 1) * 8));
    unsigned long long total = 0;
    if (nc) {
      CK(cudaMemsetAsync(ctx->work.p, 0, 16, s));
      a.mode = 1;
      a.pair_count = ctx->pair_count.as<uint32_t>();
      a.work = ctx->work.as<uint32_t>();
      if (pp::launch_scan(a, 0, 1, ctx->sm_count, nullptr, s)) return fail(ctx, PP_ERR_CUDA, "pair count launch failed");
      const uint64_t tmp_elems = (uint64_t)(nc + 1) / 2048 + 64;
      CK(ctx->scan_tmp.ensure(tmp_elems * 8 * 2));
      // offsets: exclusive scan of counts, plus the total in slot nc
      DevBuf cnt1;
      CK(cnt1.ensure(((uint64_t)nc + 1) * 4));
      CK(cudaMemcpyAsync(cnt1.p, ctx->pair_count.p, (uint64_t)nc * 4, cudaMemcpyDeviceToDevice, s));
      CK(cudaMemsetAsync(cnt1.as<uint32_t>() + nc, 0, 4, s));
      pp::launch_exclusive_scan_u64_from_u32(cnt1.as<uint32_t>(), (uint64_t)nc + 1,
                                             ctx->pair_off.as<unsigned long long>(),
                                             ctx->scan_tmp.as<unsigned long long>(), tmp_elems * 2, s);
      CK(cudaMemcpyAsync(&total, ctx->pair_off.as<unsigned long long>() + nc, 8, cudaMemcpyDeviceToHost, s));
      CK(ctx->maxlist.ensure(4));
      CK(cudaMemsetAsync(ctx->maxlist.p, 0, 4, s));
      pp::launch_max_u32(ctx->pair_count.as<uint32_t>(), nc, ctx->maxlist.as<uint32_t>(), s);
      CK(cudaMemcpyAsync(&ctx->geo_maxlist, ctx->maxlist.p, 4, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
    ctx->geo_emitted_all = false;
    ctx->geo_cloud = cloud;
    ctx->geo_key_version = cl->grid_version;
    ctx->geo_R = R;
    ctx->geo_H = P.H;
    ctx->geo_rmin = ctx->tab.rmin;
    ctx->geo_rincr = ctx->tab.rincr;
    ctx->geo_ncentres = nc;
    ctx->geo_pairs = total;
  }
  const uint32_t nc = ctx->geo_ncentres;
  const unsigned long long total = ctx->geo_pairs;
  // ---- pair lists: all at once when they fit, else per chunk of centres
  // (each chunk's lists are emitted, then every realisation is applied)
  uint64_t cap = ctx->pair_cap_opt;
  if (!cap) {
    size_t freeb = 0, totb = 0;
    CK(cudaMemGetInfo(&freeb, &totb));
    const uint64_t held = ctx->pair_slot.bytes + ctx->pair_cat.bytes;
    const uint64_t reserve = (uint64_t)n * nreal * 3 + (uint64_t)nc * nreal * 3 + (4ull << 30);
    const uint64_t avail = freeb + held > reserve ? freeb + held - reserve : 0;
    cap = avail / 6 * 7 / 10;
  }
  cap = std::max<uint64_t>(cap, std::max<uint64_t>(ctx->geo_maxlist, 1));
  const bool chunked = total > cap;
  const uint64_t list_len = chunked ? cap : total;
  CK(ctx->pair_slot.ensure(std::max<uint64_t>(list_len, 1) * 4));
  CK(ctx->pair_cat.ensure(std::max<uint64_t>(list_len, 1) * 2));
  pp::ScanArgs ea;  // the emit pass (category-sorted lists of a range of centres)
  std::memset(&ea, 0, sizeof ea);
  fill_scan_common(ea, *cl, P, D, ctx->tab);
  ea.labels = cl->label_sorted.as<uint8_t>();
  ea.flags = 0;
  CK(ctx->geo_counters.ensure(16));
  ea.counters = ctx->geo_counters.as<unsigned long long>();
  ea.status = ctx->res.status.as<int>();
  ea.rdf_in_smem = 0;
  ea.mode = 2;
  ea.pair_slot = ctx->pair_slot.as<uint32_t>();
  ea.pair_cat = ctx->pair_cat.as<uint16_t>();
  CK(ctx->work.ensure(16));
  ea.work = ctx->work.as<uint32_t>() + 2;
  const pp::ScanArgs ea_sig = ea;  // before any range is set: the graph's key
  auto set_emit_range = [&](uint32_t c0, uint32_t c1, unsigned long long p0, unsigned long long p1) {
    ea.centres = ctx->geo_centres.as<uint32_t>() + c0;
    ea.ncentres = c1 - c0;
    ea.pair_off = ctx->pair_off.as<unsigned long long>() + c0;
    ea.pair_base = p0;
    ea.pair_cap = p1 - p0;
  };
  if (!chunked && !ctx->geo_emitted_all && nc) {
    set_emit_range(0, nc, 0, total);
    CK(cudaMemsetAsync(ea.work, 0, 4, s));
    if (pp::launch_scan(ea, 0, 1, ctx->sm_count, nullptr, s)) return fail(ctx, PP_ERR_CUDA, "pair emit launch failed");
    CK(cudaGetLastError());
    ctx->geo_emitted_all = true;
  }
  if (chunked) ctx->geo_emitted_all = false;
  struct Chunk { uint32_t c0, c1; unsigned long long p0, p1; };
  std::vector<Chunk> chunks;
  if (!chunked) {
    chunks.push_back({0, nc, 0, total});
  } else {
    auto off = [&](uint32_t i, unsigned long long* v) {
      return cudaMemcpy(v, ctx->pair_off.as<unsigned long long>() + i, 8, cudaMemcpyDeviceToHost);
    };
    uint32_t c = 0;
    unsigned long long pc = 0;
    while (c < nc) {
      // the last centre c1 with pair_off[c1] - pair_off[c] <= cap
      uint32_t lo = c + 1, hi = nc;
      while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        unsigned long long v = 0;
        CK(off(mid, &v));
        if (v - pc <= cap) lo = mid; else hi = mid - 1;
      }
      unsigned long long pe = 0;
      CK(off(lo, &pe));
      chunks.push_back({c, lo, pc, pe});
      c = lo;
      pc = pe;
    }
  }
  // ---- realisation labels (sorted-slot order) and centre masks
  CK(ctx->real_labels.ensure(std::max<uint64_t>(n, 1) * nreal));
  CK(ctx->centre_ok.ensure(std::max<uint64_t>(nc, 1) * nreal));
  int r = 0;
  uint8_t* RL = ctx->real_labels.as<uint8_t>();
  uint8_t* OK = ctx->centre_ok.as<uint8_t>();
  if (include_original) {
    CK(cudaMemcpyAsync(RL, cl->label_sorted.p, n, cudaMemcpyDeviceToDevice, s));
    pp::launch_perm_mask(RL, ctx->geo_centres.as<uint32_t>(), nc, D.cslot, OK, s);
    ++r;
  }
  if (n_label_sets) {
    cudaPointerAttributes attr{};
    const bool on_dev = cudaPointerGetAttributes(&attr, label_sets) == cudaSuccess && attr.type == cudaMemoryTypeDevice;
    cudaGetLastError();
    const uint8_t* src = label_sets;
    if (!on_dev) {
      CK(ctx->gather_src.ensure(std::max<uint64_t>(n, 1) * n_label_sets));
      CK(cudaMemcpyAsync(ctx->gather_src.p, label_sets, n * (uint64_t)n_label_sets, cudaMemcpyHostToDevice, s));
      src = ctx->gather_src.as<uint8_t>();
    }
    pp::launch_gather_labels(src, cl->id_of_slot.as<uint32_t>(), n, RL + (uint64_t)r * n, n_label_sets, s);
    for (int q = 0; q < n_label_sets; ++q)
      pp::launch_perm_mask(RL + (uint64_t)(r + q) * n, ctx->geo_centres.as<uint32_t>(), nc, D.cslot,
                           OK + (uint64_t)(r + q) * nc, s);
    r += n_label_sets;
  }
  if (n_rois) {
    for (int q = 0; q < n_rois; ++q)
      CK(cudaMemcpyAsync(RL + (uint64_t)(r + q) * n, cl->label_sorted.p, n, cudaMemcpyDeviceToDevice, s));
    CK(ctx->rois_dev.ensure((size_t)n_rois * 16));
    CK(cudaMemcpyAsync(ctx->rois_dev.p, rois, (size_t)n_rois * 16, cudaMemcpyHostToDevice, s));
    pp::launch_roi_mask(cl->ions.as<float4>(), ctx->geo_centres.as<uint32_t>(), nc, ctx->rois_dev.as<float>(), n_rois,
                        R, cl->label_sorted.as<uint8_t>(), D.cslot, OK + (uint64_t)r * nc, s);
    r += n_rois;
  }
  CK(cudaGetLastError());
  // ---- apply every realisation: one persistent launch for RDF and the
  // per-realisation counts, plus the 32-realisation kNN walk/bin launches,
  // all captured once into a CUDA graph
  if (nc) {
    CK(ctx->work.ensure(16));
    pp::ApplyArgs b;
    std::memset(&b, 0, sizeof b);
    b.centres = ctx->geo_centres.as<uint32_t>();
    b.ncentres = nc;
    b.nc_total = nc;
    b.pair_off = ctx->pair_off.as<unsigned long long>();
    b.pair_slot = ctx->pair_slot.as<uint32_t>();
    b.pair_cat = ctx->pair_cat.as<uint16_t>();
    b.n = n;
    b.nreal = nreal;
    b.H = P.H;
    b.cat_miss = P.cat_miss;
    b.cslot_of = D.cslot;
    b.eslot_of = D.eslot;
    b.nC = P.nC;
    b.nE = P.nE;
    b.envbits = D.envbits;
    b.set_list = D.set_list;
    b.nsets = D.nsets;
    b.nS = P.nS;
    b.kvals = D.kvals;
    b.nkI = (int)P.kvals.size();
    b.kmax = std::max(P.kmax, 1);
    b.flags = ((flags & (PP_RDF | PP_RIPK)) ? PP_RDF : 0) | (P.kr ? PP_MKNN : 0);
    b.rdf_core = ctx->res.rdf.as<unsigned long long>();
    b.knn_core = ctx->res.knn.as<unsigned long long>();
    b.counters = ctx->res.counters.as<unsigned long long>();
    b.work = ctx->work.as<uint32_t>();
    b.status = ctx->res.status.as<int>();
    b.nsmax = std::max(P.emax, 1);
    b.disjoint = P.disjoint;
    b.setidx = D.setidx;
    b.count = 1;
    // kNN of 32 realisations per warp (walk + bin) where its records and bins
    // fit; the fused kernel then does RDF and the per-realisation counters
    pp::KnnArgs kq;
    std::memset(&kq, 0, sizeof kq);
    bool knn32 = false;
    if (b.flags & PP_MKNN) {
      kq.centres = b.centres;
      kq.ncentres = nc;
      kq.pair_off = b.pair_off;
      kq.pair_slot = b.pair_slot;
      kq.pair_cat = b.pair_cat;
      kq.n = n;
      kq.nreal = nreal;
      kq.cslot_of = D.cslot;
      kq.envbits = D.envbits;
      kq.disjoint = P.disjoint;
      kq.setidx = D.setidx;
      kq.nsets = D.nsets;
      kq.set_list = D.set_list;
      kq.kvals = D.kvals;
      kq.nkI = b.nkI;
      kq.kmax = b.kmax;
      kq.nsmax = b.nsmax;
      kq.nC = P.nC;
      kq.nS = P.nS;
      kq.H = P.H;
      kq.cat_miss = P.cat_miss;
      kq.knn_core = b.knn_core;
      knn32 = pp::knn32_check(kq) == 0;
      if (knn32) b.flags &= ~PP_MKNN;
    }
    if (pp::apply_configure(b)) return fail(ctx, PP_ERR_UNSUPPORTED, "RDF bins of one realisation exceed shared memory");
    b.ngroups = (nreal + b.group - 1) / b.group;
    // tile: enough pairs per item to amortise the per-item flush of the
    // shared bins, enough items to balance the persistent blocks, at most
    // 65535 centres (16-bit kNN bins) and fewer than 2^31 pairs (RDF bins)
    {
      const double avg = std::max((double)ctx->geo_pairs / std::max<uint32_t>(nc, 1), 1.0);
      const double flush_words = ((b.flags & PP_RDF) ? (double)P.nC * P.nE * P.H * b.group : 0.0) +
                                 (b.knn_smem ? (double)P.nC * P.nS * P.kvals.size() * P.H * b.group / 2 : 0.0);
      double tile = std::max(1.0e6, 256.0 * flush_words) / (avg * b.group);
      const double balance = (double)nc * b.ngroups / (8.0 * ctx->sm_count);
      tile = std::min(tile, balance);
      tile = std::min(tile, 2147483647.0 / std::max<uint32_t>(ctx->geo_maxlist, 1));
      tile = std::min(tile, 65535.0);
      b.tile = (uint32_t)std::max(32.0, std::floor(tile));
      if ((double)b.tile * ctx->geo_maxlist >= 2147483648.0 && b.tile > 1)
        b.tile = (uint32_t)std::max<uint64_t>(1, 2147483647ull / std::max<uint32_t>(ctx->geo_maxlist, 1));
    }
    const uint64_t nrg = (uint64_t)b.ngroups * b.group;
    CK(ctx->labels_il.ensure(std::max<uint64_t>(n, 1) * nrg));
    CK(ctx->ok_il.ensure(std::max<uint64_t>(nc, 1) * nrg));
    pp::launch_interleave(RL, nreal, n, b.group, ctx->labels_il.as<uint8_t>(), s);
    pp::launch_interleave(OK, nreal, nc, b.group, ctx->ok_il.as<uint8_t>(), s);
    b.labels = ctx->labels_il.as<uint8_t>();
    b.centre_ok = ctx->ok_il.as<uint8_t>();
    int ng32 = 0;
    uint32_t chunk = 0;
    const uint64_t NT = (uint64_t)kq.nsmax * kq.nkI;
    // a few realisations beyond the last full group of 32 take the rank walk
    // of the fused kernel in a launch of their own (a 32-lane group of them
    // would leave most lanes idle)
    pp::ApplyArgs bk;
    std::memset(&bk, 0, sizeof bk);
    bool knn_rest = false;
    if (knn32) {
      const int rest = nreal % 32;
      ng32 = (nreal + 31) / 32;
      if (rest > 0 && rest <= 8) {
        bk = b;
        bk.flags = PP_MKNN;
        bk.count = 0;
        bk.rbase = nreal - rest;
        bk.nreal = rest;
        if (pp::apply_configure(bk) == 0) {
          knn_rest = true;
          ng32 = nreal / 32;
          bk.ngroups = (rest + bk.group - 1) / bk.group;
          bk.tile = b.tile;
          const uint64_t nrk = (uint64_t)bk.ngroups * bk.group;
          CK(ctx->knn_rest_labels.ensure(std::max<uint64_t>(n, 1) * nrk));
          CK(ctx->knn_rest_ok.ensure(std::max<uint64_t>(nc, 1) * nrk));
          pp::launch_interleave(RL + (uint64_t)bk.rbase * n, rest, n, bk.group, ctx->knn_rest_labels.as<uint8_t>(), s);
          pp::launch_interleave(OK + (uint64_t)bk.rbase * nc, rest, nc, bk.group, ctx->knn_rest_ok.as<uint8_t>(), s);
          bk.labels = ctx->knn_rest_labels.as<uint8_t>();
          bk.centre_ok = ctx->knn_rest_ok.as<uint8_t>();
        }
      }
      // the realisations of the 32-lane groups (all, or all but the rest)
      const uint64_t r32 = std::min<uint64_t>((uint64_t)ng32 * 32, (uint64_t)nreal);
      CK(ctx->knn_labels.ensure(std::max<uint64_t>(n, 1) * 32 * std::max(ng32, 1)));
      CK(ctx->knn_ok.ensure(std::max<uint64_t>(nc, 1) * 32 * std::max(ng32, 1)));
      if (r32) {
        pp::launch_interleave(RL, r32, n, 32, ctx->knn_labels.as<uint8_t>(), s);
        pp::launch_interleave(OK, r32, nc, 32, ctx->knn_ok.as<uint8_t>(), s);
      }
      kq.labels = ctx->knn_labels.as<uint8_t>();
      kq.centre_ok = ctx->knn_ok.as<uint8_t>();
      // records of one launch: at most 3 GiB
      const uint64_t per_centre = NT * 64 + 32;
      chunk = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(nc, (3ull << 30) / per_centre));
      CK(ctx->knn_rec.ensure((uint64_t)chunk * NT * 64));
      CK(ctx->knn_recc.ensure((uint64_t)chunk * 32));
      kq.rec = ctx->knn_rec.as<uint16_t>();
      kq.rec_c = ctx->knn_recc.as<uint8_t>();
      kq.work = ctx->work.as<uint32_t>() + 1;
    }
    auto enqueue = [&](cudaStream_t st) -> int {
      for (const Chunk& ch : chunks) {
        if (chunked) {
          set_emit_range(ch.c0, ch.c1, ch.p0, ch.p1);
          if (cudaMemsetAsync(ea.work, 0, 4, st) != cudaSuccess) return fail(ctx, PP_ERR_CUDA, "memset failed");
          if (pp::launch_scan(ea, 0, 1, ctx->sm_count, nullptr, st)) return fail(ctx, PP_ERR_CUDA, "pair emit launch failed");
        }
        pp::ApplyArgs bc = b;
        bc.centres = b.centres + ch.c0;
        bc.ncentres = ch.c1 - ch.c0;
        bc.pair_off = b.pair_off + ch.c0;
        bc.cbase = ch.c0;
        bc.pair_base = ch.p0;
        if (cudaMemsetAsync(ctx->work.p, 0, 8, st) != cudaSuccess) return fail(ctx, PP_ERR_CUDA, "memset failed");
        if (pp::launch_apply(bc, ctx->sm_count, st)) return fail(ctx, PP_ERR_CUDA, "apply launch failed");
        if (knn_rest) {
          pp::ApplyArgs kc = bk;
          kc.centres = bk.centres + ch.c0;
          kc.ncentres = ch.c1 - ch.c0;
          kc.pair_off = bk.pair_off + ch.c0;
          kc.cbase = ch.c0;
          kc.pair_base = ch.p0;
          kc.work = ctx->work.as<uint32_t>() + 3;
          if (cudaMemsetAsync(kc.work, 0, 4, st) != cudaSuccess) return fail(ctx, PP_ERR_CUDA, "memset failed");
          if (pp::launch_apply(kc, ctx->sm_count, st)) return fail(ctx, PP_ERR_CUDA, "kNN rest launch failed");
        }
        pp::KnnArgs k = kq;
        k.pair_base = ch.p0;
        for (int g = 0; g < ng32; ++g) {
          for (uint32_t c0 = ch.c0; c0 < ch.c1; c0 += chunk) {
            k.grp = g;
            k.c0 = c0;
            k.cn = std::min(chunk, ch.c1 - c0);
            k.tile = 4;  // centres per warp work item
            if (cudaMemsetAsync(k.work, 0, 4, st) != cudaSuccess) return fail(ctx, PP_ERR_CUDA, "memset failed");
            if (pp::launch_knn_walk(k, ctx->sm_count, st)) return fail(ctx, PP_ERR_CUDA, "kNN walk launch failed");
            const uint32_t nranges = (uint32_t)std::max<uint64_t>(1, (8ull * ctx->sm_count + NT - 1) / NT);
            k.tile = std::max<uint32_t>(1, (k.cn + nranges - 1) / nranges);
            if (cudaMemsetAsync(k.work, 0, 4, st) != cudaSuccess) return fail(ctx, PP_ERR_CUDA, "memset failed");
            if (pp::launch_knn_bin(k, ctx->sm_count, st)) return fail(ctx, PP_ERR_CUDA, "kNN bin launch failed");
          }
        }
      }
      return PP_OK;
    };
    std::string sig((const char*)&b, sizeof b);
    sig.append((const char*)&kq, sizeof kq);
    sig.append((const char*)&ea_sig, sizeof ea_sig);
    sig.append((const char*)&bk, sizeof bk);
    sig.append((const char*)chunks.data(), chunks.size() * sizeof(Chunk));
    const uint64_t extra[5] = {(uint64_t)ng32, chunk, nc, (uint64_t)ctx->sm_count, chunked ? 1u : 0u};
    sig.append((const char*)extra, sizeof extra);
    if (!ctx->apply_exec || sig != ctx->apply_sig) {
      if (!ctx->cap_stream) CK(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
      if (ctx->apply_exec) {
        cudaGraphExecDestroy(ctx->apply_exec);
        ctx->apply_exec = nullptr;
      }
      ctx->apply_sig.clear();
      CK(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeRelaxed));
      const int erc = enqueue(ctx->cap_stream);
      cudaGraph_t graph = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(ctx->cap_stream, &graph);
      if (erc) {
        if (graph) cudaGraphDestroy(graph);
        return erc;
      }
      CK(ce);
      size_t nodes = 0;
      cudaGraphGetNodes(graph, nullptr, &nodes);
      const cudaError_t ie = cudaGraphInstantiate(&ctx->apply_exec, graph, 0);
      cudaGraphDestroy(graph);
      CK(ie);
      ctx->apply_sig = sig;
      ctx->graph_nodes = nodes;
      ++ctx->graph_captures;
    }
    CK(cudaEventRecord(ctx->ev0, s));
    CK(cudaGraphLaunch(ctx->apply_exec, s));
    CK(cudaEventRecord(ctx->ev1, s));
    ++ctx->graph_launches;
    ctx->ev_recorded = true;
  }
  ctx->res.valid = true;
  return PP_OK;
}

int pp_kernel_launches(uint64_t* count) {
  if (!count) return PP_ERR_INVALID;
  *count = pp::kernel_launches();
  return PP_OK;
}

int pp_last_kernel_ms(pp_ctx* ctx, float* ms) {
  if (!ctx || !ms) return PP_ERR_INVALID;
  if (!ctx->ev_recorded) { *ms = 0.f; return PP_OK; }
  CK(cudaEventSynchronize(ctx->ev1));
  CK(cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
  return PP_OK;
}

int pp_run_tests(pp_ctx* ctx, uint64_t* tests) {
  if (!ctx || !tests) return PP_ERR_INVALID;
  if (!ctx->res.valid || ctx->res.batched) return fail(ctx, PP_ERR_STATE, "no plain run");
  CK(cudaStreamSynchronize(ctx->res.stream));
  unsigned long long t = 0;
  CK(cudaMemcpy(&t, ctx->res.tests.p, 8, cudaMemcpyDeviceToHost));
  *tests = t;
  return PP_OK;
}

int pp_last_kernel(pp_ctx* ctx, const char** name) {
  if (!ctx || !name) return PP_ERR_INVALID;
  static const char* names[] = {"k_scan", "k_brick", "k_lanes", "k_lanes_knn", "k_lanes+k_lanes_knn",
                                "k_lanes+k_scan"};
  *name = names[ctx->last_kind < 0 || ctx->last_kind > 5 ? 0 : ctx->last_kind];
  return PP_OK;
}

int pp_batched_count(pp_ctx* ctx, int* n) {
  if (!ctx || !n || !ctx->res.valid || !ctx->res.batched) return fail(ctx, PP_ERR_STATE, "no batched run");
  *n = ctx->res.nreal;
  return PP_OK;
}

int pp_fetch_batched(pp_ctx* ctx, int r, uint64_t* bins, size_t cap) {
  if (!ctx || !ctx->res.valid || !ctx->res.batched) return fail(ctx, PP_ERR_STATE, "no batched run");
  if (r < 0 || r >= ctx->res.nreal) return fail(ctx, PP_ERR_INVALID, "bad realisation");
  int rc = fetch_cores(ctx);
  if (rc) return rc;
  const uint64_t need = result_len(ctx->res);
  if (!bins || cap < need) return fail(ctx, PP_ERR_INVALID, "result needs %llu uint64", (unsigned long long)need);
  finalize(ctx->res, r, bins);
  return PP_OK;
}

int pp_batched_stats(pp_ctx* ctx, int r, uint64_t* centres, uint64_t* pairs) {
  if (!ctx || !ctx->res.valid || !ctx->res.batched) return fail(ctx, PP_ERR_STATE, "no batched run");
  if (r < 0 || r >= ctx->res.nreal) return fail(ctx, PP_ERR_INVALID, "bad realisation");
  int rc = fetch_cores(ctx);
  if (rc) return rc;
  if (pairs) *pairs = ctx->res.counters_h[2 * r];
  if (centres) *centres = ctx->res.counters_h[2 * r + 1];
  return PP_OK;
}

int pp_batched_graph(pp_ctx* ctx, uint64_t* nodes, uint64_t* captures, uint64_t* launches) {
  if (!ctx) return PP_ERR_INVALID;
  if (nodes) *nodes = ctx->graph_nodes;
  if (captures) *captures = ctx->graph_captures;
  if (launches) *launches = ctx->graph_launches;
  return PP_OK;
}

}  // extern "C"

// ================================================================ serving
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ServerRequest {
  uint64_t ticket = 0;
  int cloud = -1;
  bool mergeable = false;  // may share a merged pass with other queries of its cloud
  uint32_t flags = 0;
  float rmin = 0, rincr = 0, rmax = 0;
  std::vector<uint32_t> trg, env, ks;
  int ntasks = 0;
  uint64_t footprint = 0;
  int rc = PP_OK;
  std::string err;
  std::vector<uint64_t> bins;
  bool dense = false;       // centres dense enough for the centre-per-lane scans (runs alone)
  uint64_t pairs = 0, centres = 0;
  double t_submit = 0, t_end = 0;
  bool done = false;
};

}  // namespace

struct pp_server {
  pp_ctx* ctx = nullptr;
  std::vector<pp_ctx*> workers;
  std::vector<cudaStream_t> streams;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_queue, cv_done;
  std::deque<std::shared_ptr<ServerRequest>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<ServerRequest>> reqs;
  uint64_t next_ticket = 1;
  uint64_t budget = 0, inflight = 0;
  bool stop = false;
  uint64_t submitted = 0, admitted = 0, rejected = 0, completed = 0, batches = 0;
  int max_batch = pp::kMultiMaxQueries;  // queries per merged pass (option "server_batch")
  double pairs_done = 0;
  std::vector<double> latencies;
};

namespace {

// One query on a worker context: the plain path on the worker's stream.
void serve_one(pp_ctx* w, cudaStream_t st, ServerRequest& q) {
  int rc = pp_tasks_set(w, q.trg.data(), q.env.data(), q.ntasks);
  if (!rc) rc = pp_hist_params(w, q.rmin, q.rincr, q.rmax);
  if (!rc) rc = pp_run(w, q.cloud, q.flags, q.ks.empty() ? nullptr : q.ks.data(), (int)q.ks.size(), nullptr, st);
  uint64_t total = 0, nb = 0;
  if (!rc) rc = pp_result_size(w, &total, &nb);
  if (!rc) {
    q.bins.assign(std::max<uint64_t>(total, 1), 0);
    rc = pp_fetch(w, q.bins.data(), q.bins.size());
    q.bins.resize(total);
  }
  if (!rc) rc = pp_run_stats(w, nullptr, nullptr, &q.pairs);
  q.rc = rc;
  if (rc) q.err = w->err;
}

// Several queries on one cloud in one merged pass (k_multi): each keeps its
// own radius, histogram geometry, hull-distance test, tasks and kNN orders,
// and gets the bins, pairs and centres it would get alone through pp_run.
// Sets rc, bins and pairs of every request.
void run_multi(pp_ctx* w, const std::vector<ServerRequest*>& qs, cudaStream_t s) {
  auto fail_all = [&](int rc) {
    for (ServerRequest* r : qs) {
      r->rc = rc;
      r->err = w->err;
    }
  };
  Cloud* cl = get_cloud(w, qs[0]->cloud);
  const int nq = (int)qs.size();
  if (!cl || nq < 1 || nq > pp::kMultiMaxQueries) return fail_all(fail(w, PP_ERR_INVALID, "bad merged batch"));
  const uint64_t n = cl->n;
  struct Prep {
    Tables t;
    std::vector<float> T;
    std::vector<uint16_t> lut;
    int shift = 0;
    uint32_t base = 0;
    std::vector<uint32_t> kvals;
    float rp = 0.f;
  };
  std::vector<Prep> P(nq);
  std::vector<pp::MultiQuery> MQ(nq);
  std::vector<pp::MultiTask> MT;
  std::vector<uint32_t> q_of_type(256, 0u);
  std::vector<unsigned long long> t_of_type(256, 0ull), env_of_type(256, 0ull), t_of_q(nq, 0ull);
  unsigned long long rdf_tasks = 0, knn_tasks = 0;
  std::vector<float> Tall;
  std::vector<uint16_t> Lall;
  std::vector<int> Kall;
  uint64_t rdf_words = 0, knn_words = 0;
  float Rmax = 0.f;
  for (int q = 0; q < nq; ++q) {
    const ServerRequest& r = *qs[q];
    Prep& p = P[q];
    set_tables(p.t, r.rmin, r.rincr, r.rmax);
    if (p.t.nbins == 0 || p.t.nbins + 2 > 16384) return fail_all(fail(w, PP_ERR_INVALID, "query histogram"));
    p.T = threshold_table(p.t);
    build_lut(p.T, p.t.rmax * p.t.rmax, 4096, p.lut, p.shift, p.base);
    std::vector<uint32_t> ks;
    if (r.flags & PP_MKNN) ks = r.ks;
    if (r.flags & PP_1NN) ks.push_back(1);
    std::sort(ks.begin(), ks.end());
    ks.erase(std::unique(ks.begin(), ks.end()), ks.end());
    p.kvals = ks;
    const float R = p.t.rmax;
    Rmax = std::max(Rmax, R);
    pp::MultiQuery& Q = MQ[q];
    Q.R = R;
    Q.R2 = R * R;
    const float Rm = R + cl->g.margin;
    Q.Rm2 = Rm * Rm;
    Q.H = (int)p.t.nbins + 2;
    Q.cat_miss = category_of_distance(p.t, (float)((double)R + kEpsilon));
    Q.lut_n = (int)p.lut.size();
    Q.lut_shift = p.shift;
    Q.lut_base = p.base;
    Q.T_off = (uint32_t)Tall.size();
    Q.lut_off = (uint32_t)Lall.size();
    Q.kv_off = (uint32_t)Kall.size();
    Q.nkI = (int)ks.size();
    Q.kmax = ks.empty() ? 0 : (int)ks.back();
    Tall.insert(Tall.end(), p.T.begin(), p.T.end());
    Lall.insert(Lall.end(), p.lut.begin(), p.lut.end());
    for (uint32_t k : ks) Kall.push_back((int)k);
    for (int k = 0; k < r.ntasks; ++k) {
      const int t = (int)MT.size();
      if (t >= pp::kMultiMaxTasks) return fail_all(fail(w, PP_ERR_INVALID, "too many tasks in a merged batch"));
      pp::MultiTask T{};
      T.q = q;
      T.rdf = 0xffffffffu;
      T.knn = 0xffffffffu;
      if (r.flags & (PP_RDF | PP_RIPK)) {
        T.rdf = (uint32_t)rdf_words;
        rdf_words += (uint64_t)Q.H;
        rdf_tasks |= 1ull << t;
      }
      if (!ks.empty()) {
        T.knn = (uint32_t)knn_words;
        knn_words += (uint64_t)Q.H * ks.size();
        knn_tasks |= 1ull << t;
      }
      for (int ty = 0; ty < 256; ++ty) {
        if (has_type(&r.trg[8 * k], ty)) {
          t_of_type[ty] |= 1ull << t;
          q_of_type[ty] |= 1u << q;
        }
        if (has_type(&r.env[8 * k], ty)) env_of_type[ty] |= 1ull << t;
      }
      t_of_q[q] |= 1ull << t;
      MT.push_back(T);
    }
  }
  int lists = 0;
  for (int ty = 0; ty < 256; ++ty) lists = std::max(lists, __builtin_popcountll(t_of_type[ty] & knn_tasks));
  // the cloud's grid serves radii up to 6 cell edges (its stencil tables)
  if (!cl->grid_ok || Rmax > cl->g.h * 6.f)
    return fail_all(fail(w, PP_ERR_STATE, "cloud was not prepared for R = %g (pp_cloud_prepare)", (double)Rmax));
  // hull-distance groups: queries sharing R' = max(R, carve) share one ion2surf
  std::vector<float> grp_rp;
  std::vector<int> grp_of(nq, 0);
  for (int q = 0; q < nq; ++q) {
    const float rp = cl->has_user_surf ? -1.f : std::max(P[q].t.rmax, cl->hull.carve);
    int g = 0;
    while (g < (int)grp_rp.size() && grp_rp[g] != rp) ++g;
    if (g == (int)grp_rp.size()) grp_rp.push_back(rp);
    grp_of[q] = g;
  }
  std::vector<float> grpR2;
  std::vector<uint32_t> grpBits;
  std::vector<int> grp_off(grp_rp.size() + 1, 0);
  for (size_t g = 0; g < grp_rp.size(); ++g) {
    grp_off[g] = (int)grpR2.size();
    for (int q = 0; q < nq; ++q)
      if (grp_of[q] == (int)g) {
        grpR2.push_back(MQ[q].R2);
        grpBits.push_back(1u << q);
      }
  }
  grp_off[grp_rp.size()] = (int)grpR2.size();
  // tables in one device block
  std::vector<unsigned char> blob;
  auto put = [&](const void* src, size_t bytes) {
    size_t off = (blob.size() + 15) & ~size_t(15);
    blob.resize(off + bytes);
    if (bytes) std::memcpy(blob.data() + off, src, bytes);
    return off;
  };
  int nrow = 0;
  const int8_t* rows = pp::row_table_host(&nrow);
  const size_t oQ = put(MQ.data(), MQ.size() * sizeof(pp::MultiQuery));
  const size_t oT = put(MT.data(), MT.size() * sizeof(pp::MultiTask));
  const size_t oqt = put(q_of_type.data(), 256 * 4);
  const size_t ott = put(t_of_type.data(), 256 * 8);
  const size_t oet = put(env_of_type.data(), 256 * 8);
  const size_t otq = put(t_of_q.data(), t_of_q.size() * 8);
  const size_t oTa = put(Tall.data(), Tall.size() * 4);
  const size_t oL = put(Lall.data(), Lall.size() * 2);
  const size_t oK = put(Kall.data(), std::max<size_t>(Kall.size(), 1) * 4);
  const size_t oR = put(grpR2.data(), grpR2.size() * 4);
  const size_t oB = put(grpBits.data(), grpBits.size() * 4);
  const size_t orow = put(rows, (size_t)nrow * 2);
  const uint64_t core_words = std::max<uint64_t>(rdf_words + knn_words, 1);
  if (w->tables_dev.ensure(blob.size()) != cudaSuccess || w->multi_cmask.ensure(std::max<uint64_t>(n, 1) * 4) != cudaSuccess ||
      w->multi_cores.ensure(core_words * 8 + 16 * pp::kMultiMaxQueries + 16) != cudaSuccess ||
      w->centres.ensure(std::max<uint64_t>(n, 1) * 4) != cudaSuccess || w->centre_count.ensure(8) != cudaSuccess ||
      w->sel_flags.ensure((n + 1) * 4) != cudaSuccess)
    return fail_all(fail(w, PP_ERR_NOMEM, "device allocation for a merged pass failed"));
  const uint64_t tmp_elems = (n + 1) / 2048 + 64;
  if (w->sel_tmp.ensure(tmp_elems * 4 * 2) != cudaSuccess || w->work.ensure(32) != cudaSuccess)
    return fail_all(fail(w, PP_ERR_NOMEM, "device allocation for a merged pass failed"));
  unsigned char* b = w->tables_dev.as<unsigned char>();
  unsigned long long* cores = w->multi_cores.as<unsigned long long>();
  unsigned long long* counters = cores + core_words;
  int* status = reinterpret_cast<int*>(counters + 2 * pp::kMultiMaxQueries);
  uint32_t* cmask = w->multi_cmask.as<uint32_t>();
  auto ck = [&](cudaError_t e) { return e == cudaSuccess; };
  if (!ck(cudaMemcpyAsync(b, blob.data(), blob.size(), cudaMemcpyHostToDevice, s)) ||
      !ck(cudaMemsetAsync(cores, 0, core_words * 8 + 16 * pp::kMultiMaxQueries + 16, s)) ||
      !ck(cudaMemsetAsync(cmask, 0, std::max<uint64_t>(n, 1) * 4, s)) || !ck(cudaMemsetAsync(w->work.p, 0, 32, s)))
    return fail_all(fail(w, PP_ERR_CUDA, "merged pass set-up failed"));
  // hull-distance bits: each group's ion2surf as a lone query computes it
  for (size_t g = 0; g < grp_rp.size(); ++g) {
    const float* surf = nullptr;
    int gq = 0;
    while (grp_of[gq] != (int)g) ++gq;
    int rc = ensure_surface(w, *cl, P[gq].t.rmax, s, &surf);
    if (rc) return fail_all(rc);
    pp::launch_cmask_or(surf, n, reinterpret_cast<const float*>(b + oR) + grp_off[g],
                        reinterpret_cast<const uint32_t*>(b + oB) + grp_off[g], grp_off[g + 1] - grp_off[g], cmask, s);
  }
  pp::launch_multi_select(cl->label_sorted.as<uint8_t>(), cmask, reinterpret_cast<const uint32_t*>(b + oqt), n,
                          w->sel_flags.as<uint32_t>(), w->sel_tmp.as<uint32_t>(), tmp_elems * 2,
                          w->centres.as<uint32_t>(), w->centre_count.as<uint32_t>(), s);
  uint32_t ncent = 0;
  if (!ck(cudaGetLastError()) || !ck(cudaMemcpyAsync(&ncent, w->centre_count.p, 4, cudaMemcpyDeviceToHost, s)) ||
      !ck(cudaStreamSynchronize(s)))
    return fail_all(fail(w, PP_ERR_CUDA, "merged pass centre selection failed"));
  if (ncent > 0) {
    pp::MultiArgs m{};
    pp::ScanArgs& a = m.s;
    a.ions = cl->ions.as<float4>();
    a.cell_start = cl->cell_start.as<uint32_t>();
    a.g = cl->g;
    a.labels = cl->label_sorted.as<uint8_t>();
    a.rowtab = reinterpret_cast<const int8_t*>(b + orow);
    a.status = status;
    a.sym = 0;
    m.cmask = cmask;
    m.centres = w->centres.as<uint32_t>();
    m.ncentres = ncent;
    m.nq = nq;
    m.nt = (int)MT.size();
    m.qs = reinterpret_cast<const pp::MultiQuery*>(b + oQ);
    m.ts = reinterpret_cast<const pp::MultiTask*>(b + oT);
    m.q_of_type = reinterpret_cast<const uint32_t*>(b + oqt);
    m.t_of_type = reinterpret_cast<const unsigned long long*>(b + ott);
    m.env_of_type = reinterpret_cast<const unsigned long long*>(b + oet);
    m.t_of_q = reinterpret_cast<const unsigned long long*>(b + otq);
    m.rdf_tasks = rdf_tasks;
    m.knn_tasks = knn_tasks;
    m.T = reinterpret_cast<const float*>(b + oTa);
    m.lut = reinterpret_cast<const uint16_t*>(b + oL);
    m.kvals = reinterpret_cast<const int*>(b + oK);
    m.rdf_core = cores;
    m.knn_core = cores + rdf_words;
    m.counters = counters;
    m.rdf_words = (uint32_t)rdf_words;
    m.lists = lists;
    m.tile = 32;
    m.work = w->work.as<uint32_t>();
    size_t smem = 0;
    const int rc = pp::launch_multi(m, w->sm_count, &smem, s);
    if (rc) return fail_all(fail(w, PP_ERR_CUDA, "merged pass launch failed (%d, %zu B shared)", rc, smem));
  }
  std::vector<unsigned long long> hc(core_words + 2 * pp::kMultiMaxQueries + 2);
  if (!ck(cudaMemcpyAsync(hc.data(), cores, hc.size() * 8, cudaMemcpyDeviceToHost, s)) ||
      !ck(cudaStreamSynchronize(s)))
    return fail_all(fail(w, PP_ERR_CUDA, "merged pass failed"));
  int st = 0;
  std::memcpy(&st, &hc[core_words + 2 * pp::kMultiMaxQueries], 4);
  if (st) return fail_all(fail(w, PP_ERR_DEVICE, "merged pass: device status word 0x%x", st));
  // each query's pp_fetch layout: RDF[tasks], 1NN[tasks], RIPK[tasks], MKNN[tasks][k]
  int t0 = 0;
  for (int q = 0; q < nq; ++q) {
    ServerRequest& r = *qs[q];
    const int H = MQ[q].H;
    const std::vector<uint32_t>& kv = P[q].kvals;
    auto kidx = [&](uint32_t k) { return (size_t)(std::lower_bound(kv.begin(), kv.end(), k) - kv.begin()); };
    r.bins.clear();
    auto rdf = [&](int t) {
      const unsigned long long* c = hc.data() + MT[t].rdf;
      r.bins.insert(r.bins.end(), c, c + H);
    };
    auto knn = [&](int t, uint32_t k) {
      const unsigned long long* c = hc.data() + rdf_words + MT[t].knn + kidx(k) * H;
      r.bins.insert(r.bins.end(), c, c + H);
    };
    if (r.flags & PP_RDF) for (int k = 0; k < r.ntasks; ++k) rdf(t0 + k);
    if (r.flags & PP_1NN) for (int k = 0; k < r.ntasks; ++k) knn(t0 + k, 1);
    if (r.flags & PP_RIPK) for (int k = 0; k < r.ntasks; ++k) rdf(t0 + k);
    if (r.flags & PP_MKNN)
      for (int k = 0; k < r.ntasks; ++k)
        for (uint32_t kk : r.ks) knn(t0 + k, kk);
    r.pairs = hc[core_words + 2 * q];
    r.centres = hc[core_words + 2 * q + 1];
    r.rc = PP_OK;
    t0 += r.ntasks;
  }
}

// Footprint of a merged pass on a cloud of n ions: hull-distance bits, a
// private ion2surf, selection flags, scan partials and centre list (17 B per
// ion), plus every query's result cores.
uint64_t multi_base_bytes(uint64_t n) { return 17 * n + (1u << 20); }

void worker_loop(pp_server* S, int k) {
  pp_ctx* w = S->workers[k];
  cudaSetDevice(w->device);
  for (;;) {
    std::vector<std::shared_ptr<ServerRequest>> batch;
    uint64_t fp = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      // the head of the queue, and with it every queued query of its cloud
      // that can share its pass, as far as the budget and the pass's limits
      // allow; queries that arrived while earlier passes ran join here
      auto head_fp = [&] {
        const auto& h = S->queue.front();
        return h->mergeable ? multi_base_bytes(S->ctx->clouds[h->cloud]->n) + h->footprint : h->footprint;
      };
      S->cv_queue.wait(lk, [&] { return S->stop || (!S->queue.empty() && S->inflight + head_fp() <= S->budget); });
      if (S->queue.empty()) return;  // stop requested and nothing left
      std::shared_ptr<ServerRequest> h = S->queue.front();
      S->queue.pop_front();
      batch.push_back(h);
      if (h->mergeable) {
        fp = multi_base_bytes(S->ctx->clouds[h->cloud]->n) + h->footprint;
        int tasks = h->ntasks;
        for (auto it = S->queue.begin(); it != S->queue.end() && (int)batch.size() < S->max_batch;) {
          const auto& q = *it;
          if (q->mergeable && q->cloud == h->cloud && tasks + q->ntasks <= pp::kMultiMaxTasks &&
              S->inflight + fp + q->footprint <= S->budget) {
            fp += q->footprint;
            tasks += q->ntasks;
            batch.push_back(q);
            it = S->queue.erase(it);
          } else {
            ++it;
          }
        }
      } else {
        fp = h->footprint;
      }
      S->inflight += fp;
      S->admitted += batch.size();
      S->batches++;
    }
    if (batch[0]->mergeable) {
      std::vector<ServerRequest*> raw;
      for (auto& q : batch) raw.push_back(q.get());
      run_multi(w, raw, S->streams[k]);
    } else {
      serve_one(w, S->streams[k], *batch[0]);
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->inflight -= fp;
      const double t = now_ms();
      for (auto& q : batch) {
        q->t_end = t;
        q->done = true;
        S->completed++;
        S->pairs_done += (double)q->pairs;
        S->latencies.push_back(q->t_end - q->t_submit);
      }
    }
    S->cv_done.notify_all();
    S->cv_queue.notify_all();
  }
}

}  // namespace

extern "C" {

int pp_cloud_prepare(pp_ctx* ctx, int cloud, float r_lo, float r_hi) {
  Cloud* cl = ctx ? get_cloud(ctx, cloud) : nullptr;
  if (!cl || ctx->readonly_clouds || !(r_lo > 0.f) || !(r_hi >= r_lo) || r_hi > 6.f * r_lo)
    return fail(ctx, PP_ERR_INVALID, "need 0 < r_lo <= r_hi <= 6 r_lo on an owned cloud");
  CK(cudaSetDevice(ctx->device));
  const float keep = cl->cell_ratio;
  cl->cell_ratio = 1.0f;  // cell edge r_lo serves every R in [r_lo, 6 r_lo]
  int rc = build_grid(ctx, *cl, r_lo, 0);
  cl->cell_ratio = keep;
  if (rc) return rc;
  if (cl->hull.present && !cl->has_user_surf) {
    if ((rc = ensure_tri_bins(ctx, *cl, std::max(r_hi, cl->hull.carve), 0))) return rc;
  }
  const float* surf = nullptr;
  if ((rc = ensure_surface(ctx, *cl, r_lo, 0, &surf))) return rc;
  // passes of dense centres take the centre-per-lane scans at a 4 x 2 x 2 cell
  // block (cells of r_lo), unless the cloud was tuned already
  if (!cl->lanes_bx) {
    cl->lanes_bx = 4;
    cl->lanes_by = 2;
    cl->lanes_bz = 2;
    cl->lanes_auto = true;
  }
  // ions per type: the serving scheduler's dense / sparse split
  std::vector<uint8_t> lab(cl->n);
  CK(cudaMemcpy(lab.data(), cl->label.p, cl->n, cudaMemcpyDeviceToHost));
  cl->type_count.assign(256, 0);
  for (uint8_t t : lab) cl->type_count[t]++;
  CK(cudaDeviceSynchronize());
  return PP_OK;
}

int pp_server_create(pp_ctx* ctx, int slots, uint64_t budget_bytes, pp_server** out) {
  if (!ctx || !out || slots < 1 || slots > 64 || ctx->parent) return fail(ctx, PP_ERR_INVALID, "bad server arguments");
  CK(cudaSetDevice(ctx->device));
  auto S = new (std::nothrow) pp_server();
  if (!S) return PP_ERR_NOMEM;
  S->ctx = ctx;
  S->budget = budget_bytes;
  S->max_batch = ctx->server_batch;
  for (int k = 0; k < slots; ++k) {
    pp_ctx* w = new (std::nothrow) pp_ctx();
    cudaStream_t st = nullptr;
    if (!w || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&w->ev0) != cudaSuccess || cudaEventCreate(&w->ev1) != cudaSuccess) {
      delete w;
      pp_server_destroy(S);
      return fail(ctx, PP_ERR_CUDA, "cannot create a serving worker");
    }
    w->device = ctx->device;
    w->sm_count = ctx->sm_count;
    w->parent = ctx;
    w->readonly_clouds = true;
    w->no_sym = ctx->no_sym;
    w->no_lanes = ctx->no_lanes;
    S->workers.push_back(w);
    S->streams.push_back(st);
  }
  for (int k = 0; k < slots; ++k) S->threads.emplace_back(worker_loop, S, k);
  *out = S;
  return PP_OK;
}

int pp_server_submit(pp_server* S, int cloud, uint32_t flags, float rmin, float rincr, float rmax,
                     const uint32_t* trg_mask, const uint32_t* env_mask, int ntasks, const uint32_t* k_list, int nk,
                     uint64_t* ticket) {
  if (!S || !ticket || ntasks < 1 || !trg_mask || !env_mask || nk < 0 || (nk && !k_list)) return PP_ERR_INVALID;
  Cloud* cl = get_cloud(S->ctx, cloud);
  if (!cl || !cl->grid_ok) return PP_ERR_STATE;
  auto q = std::make_shared<ServerRequest>();
  q->cloud = cloud;
  q->flags = flags;
  q->rmin = rmin; q->rincr = rincr; q->rmax = rmax;
  q->trg.assign(trg_mask, trg_mask + 8 * (size_t)ntasks);
  q->env.assign(env_mask, env_mask + 8 * (size_t)ntasks);
  q->ntasks = ntasks;
  if (nk) q->ks.assign(k_list, k_list + nk);
  uint32_t kmax = (flags & PP_1NN) ? 1u : 0u;
  if (flags & PP_MKNN)
    for (int i = 0; i < nk; ++i) kmax = std::max(kmax, k_list[i]);
  for (int i = 0; i < nk; ++i)
    if (k_list[i] < 1) return PP_ERR_INVALID;
  // queries of plain RDF / 1NN / RIPK / MKNN with k <= 32 and at most 64
  // tasks share merged passes; the others run alone on the plain path
  q->mergeable = !(flags & ~(uint32_t)(PP_RDF | PP_1NN | PP_RIPK | PP_MKNN)) && kmax <= (uint32_t)pp::kMultiMaxK &&
                 ntasks <= pp::kMultiMaxTasks && S->max_batch > 1;
  // device footprint: a merged query adds its result cores to its pass (whose
  // own buffers the scheduler counts once per pass); a lone query its centre
  // list, flags, scan scratch, centre flags, private ion2surf, per-cell
  // prefix and result cores
  // dense centres (at least 0.35 ions of a target type per non-empty cell,
  // the rule of default_block): the plain path's centre-per-lane scans beat a
  // merged pass for such a query, so it runs alone
  {
    uint64_t cand = 0;
    if (!cl->type_count.empty())
      for (int ty = 0; ty < 256; ++ty) {
        bool t = false;
        for (int k = 0; k < ntasks; ++k) t |= has_type(&trg_mask[8 * k], ty);
        if (t) cand += cl->type_count[ty];
      }
    q->dense = cl->occupied && (double)cand >= 0.35 * (double)cl->occupied;
  }
  const double nb = (rincr > 0.f) ? std::floor(((double)rmax - (double)rmin) / (double)rincr) + 2.0 : 1.0;
  const double cores = 8.0 * nb * (double)ntasks * (3.0 + (double)nk);
  q->mergeable = q->mergeable && !q->dense;
  q->footprint = q->mergeable ? (uint64_t)cores + 4096
                              : (uint64_t)(13.0 * (double)cl->n + 4.0 * (double)cl->g.ncells + cores);
  q->t_submit = now_ms();
  const uint64_t need = q->footprint + (q->mergeable ? multi_base_bytes(cl->n) : 0);
  std::lock_guard<std::mutex> lk(S->mu);
  S->submitted++;
  if (need > S->budget) {
    S->rejected++;
    return PP_ERR_NOMEM;
  }
  q->ticket = S->next_ticket++;
  S->reqs[q->ticket] = q;
  S->queue.push_back(q);
  *ticket = q->ticket;
  S->cv_queue.notify_one();
  return PP_OK;
}

int pp_server_wait(pp_server* S, uint64_t ticket, uint64_t* bins, size_t cap, uint64_t* len, uint64_t* pairs,
                   double* latency_ms) {
  if (!S) return PP_ERR_INVALID;
  std::shared_ptr<ServerRequest> q;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return PP_ERR_INVALID;
    q = it->second;
    S->cv_done.wait(lk, [&] { return q->done; });
    S->reqs.erase(ticket);
  }
  if (len) *len = q->bins.size();
  if (pairs) *pairs = q->pairs;
  if (latency_ms) *latency_ms = q->t_end - q->t_submit;
  if (q->rc) return q->rc;
  if (bins) {
    if (cap < q->bins.size()) return PP_ERR_INVALID;
    std::memcpy(bins, q->bins.data(), q->bins.size() * 8);
  }
  return PP_OK;
}

int pp_server_stats(pp_server* S, double* st) {
  if (!S || !st) return PP_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  std::vector<double> l = S->latencies;
  std::sort(l.begin(), l.end());
  auto pct = [&](double p) {
    if (l.empty()) return 0.0;
    const size_t i = (size_t)std::min<double>((double)l.size() - 1, std::ceil(p * (double)l.size()) - 1);
    return l[i];
  };
  st[0] = (double)S->submitted;
  st[1] = (double)S->admitted;
  st[2] = (double)S->rejected;
  st[3] = (double)S->completed;
  st[4] = (double)(S->admitted - S->completed);
  st[5] = pct(0.50);
  st[6] = pct(0.99);
  st[7] = S->pairs_done;
  return PP_OK;
}

int pp_server_passes(pp_server* S, uint64_t* passes, uint64_t* queries) {
  if (!S) return PP_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  if (passes) *passes = S->batches;
  if (queries) *queries = S->admitted;
  return PP_OK;
}

void pp_server_destroy(pp_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_queue.notify_all();
  for (auto& t : S->threads) t.join();
  for (size_t k = 0; k < S->workers.size(); ++k) {
    if (S->streams[k]) cudaStreamDestroy(S->streams[k]);
    pp_destroy(S->workers[k]);
  }
  delete S;
}

}  // extern "C"
