// pp_internal.h -- structures shared by the host side of the C ABI and the
// CUDA kernels of the spatial-statistics path.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pp {

// Device status word bits (kernels never trap; they record and return).
enum StatusBits : int {
  ST_CNT_OVERFLOW = 1,     // a neighbour count exceeded the CNTNB capacity
  ST_LIST_OVERFLOW = 2,    // a pair list exceeded its allocation
  ST_BAD_SLOT = 4,         // an index left its buffer (bounds check fired)
  ST_TYPE_RANGE = 8,       // a type id had no slot where one was required
};

// Uniform cell grid over a cloud's bounding box.  Cells are stored x-fastest
// (cell = (z * ny + y) * nx + x) so the cells of one (y, z) row are
// contiguous: a row of the stencil is one contiguous run of ions.
struct Grid {
  float lox, loy, loz;   // grid origin
  float h, inv_h;        // cell edge and its reciprocal
  int nx, ny, nz;
  uint64_t ncells;
  float margin;          // conservative slack for cell-membership rounding
};

// Everything the fused stencil-scan kernel reads.  Pointers are device memory.
struct ScanArgs {
  // cloud
  const float4* ions;          // sorted by cell: x, y, z, type id (as uint bits)
  const uint32_t* cell_start;  // ncells + 1
  Grid g;
  // realisation
  const uint8_t* labels;       // type per sorted slot (plain or permuted)
  const uint32_t* centres;     // sorted slots of the centres
  uint32_t ncentres;
  // geometry of the query
  float R, R2;                 // SpatStatRadiusMax and float(R*R)
  float Rm2;                   // (R + margin)^2 for conservative row trimming
  float box_R2;                // R2 (1 + 2^-12): centre-per-lane box filter bound
  int no_box_filter;           // centre-per-lane scans stage every candidate
  // bins: categories 0 = lowest, 1..nb = bins, nb+1 = highest
  int H;                       // nb + 2
  const float* cat_T;          // [H] smallest d^2 of each category (index 0 unused)
  float guess_start, guess_scale;
  // category lookup by the high bits of d^2: cell (bits(d2) >> lut_shift) -
  // lut_base (clamped) holds the category of the cell's smallest d^2
  const uint16_t* cat_lut;
  int lut_n, lut_shift;
  uint32_t lut_base;
  int lut_one;                 // the cell's category plus at most one step is exact for d^2 <= R^2
  // brick scan: cells per brick, centres per warp batch, bricks to process;
  // the centre-per-lane scan takes blocks of bx x by x bz cells
  int bx, bcap;
  int by, bz;
  uint32_t nbricks;
  // centre-per-lane scan: stencil rows of a block, (ry, rz) offsets from
  // (yb - bsr, zb - bsr), nearest to the block first; bsr rows each side
  const int16_t* brows;
  int bsr;
  // tuning samples: centre ci (brick b) of the pass is entry ci * stride
  // (b * stride) of the full list; 0 or 1 = every entry
  uint32_t sample_stride;
  int cat_miss;                // category of the float R + EPSILON
  // type maps
  const int8_t* cslot_of;      // [256] centre slot of a type or -1
  const int8_t* eslot_of;      // [256] environment slot of a type or -1
  int nC, nE;
  const uint32_t* envbits;     // [nC][256] bit p: type is in the p-th env set of slot c
  const int* set_list;         // [nC][32] global env-set id of the p-th local set
  const int* nsets;            // [nC]
  int nS;                      // global env sets
  const int* kvals;            // [nkI] internal k list (1-based)
  int nkI, kmax;
  uint32_t flags;              // PP_RDF | PP_MKNN (1NN is k = 1) | PP_CNTNB
  // outputs (uint64 atomics)
  unsigned long long* rdf_core;  // [nC][nE][H]
  unsigned long long* knn_core;  // [nC][nS][nkI][H]
  unsigned long long* cnt_core;  // [nC][nE][cmax + 1]
  int cmax;
  unsigned long long* counters;  // [0] pairs [1] centres
  unsigned long long* tests;     // candidate distance tests of a plain pass (nullable)
  uint32_t* work;                // dynamic work counter
  int* status;
  int rdf_in_smem;
  int disjoint;                  // every type is in at most one env set per centre slot
  int emax;                      // most env sets of one centre slot (shared kNN lists)
  const int8_t* setidx;          // [nC][256] that set's local index or -1 (disjoint only)
  int uniform_sets;              // every centre slot's setidx row is the same
  int lists_mode;                // kNN lane scan lists: 0 = d^2, categories when large; 1 = d^2; 2 = categories
  uint32_t tile;                 // centres per block work item
  const int8_t* rowtab;          // stencil row offsets in distance order (row_table_offset)
  int sym;                       // symmetric pass: pairs of two centres are taken once
  const uint8_t* cflag;          // [n] 1 if the sorted slot is a centre (sym only)
  const uint32_t* nc_pre;        // [ncells + 1] exclusive prefix of non-centre ions per cell (sym only)
  // pair-list mode (batched geometry)
  int mode;                      // 0 = fused bins, 1 = count pairs, 2 = emit lists
  uint32_t* pair_count;          // [ncentres] (mode 1)
  const unsigned long long* pair_off;  // [ncentres] (mode 2)
  uint32_t* pair_slot;           // [total] (mode 2)
  uint16_t* pair_cat;            // [total] (mode 2)
  unsigned long long pair_cap;
  unsigned long long pair_base;  // pair_slot/pair_cat hold positions [pair_base, pair_base + pair_cap)
};

// Realisation pass over stored pair lists (batched null models and ROIs).
struct ApplyArgs {
  const uint32_t* centres;       // sorted slots of the geometry centres
  uint32_t ncentres;
  const unsigned long long* pair_off;  // [ncentres + 1]
  const uint32_t* pair_slot;
  const uint16_t* pair_cat;
  const uint8_t* labels;         // [ngroups][n][group] type per sorted slot
  const uint8_t* centre_ok;      // [ngroups][nc_total][group] 1 if a centre in that realisation
  uint32_t cbase, nc_total;      // this launch's centres are entries [cbase, cbase + ncentres) of nc_total
  int rbase;                     // realisation r of this launch is rbase + r of the result
  int count;                     // 1: add pair and centre counts (one launch per realisation does)
  unsigned long long pair_base;  // pair_slot/pair_cat hold list positions from pair_base on
  uint64_t n;
  int nreal;
  int group, ngroups;            // realisations per work item (1, 2, 4, 8) and the number of groups
  int knn_smem;                  // kNN bins of a work item held in shared memory
  int nsmax;                     // most environment sets of one centre type
  int H, cat_miss;
  const int8_t* cslot_of;
  const int8_t* eslot_of;
  int nC, nE;
  const uint32_t* envbits;
  const int* set_list;
  const int* nsets;
  int nS;
  const int* kvals;
  int kmax;                      // largest k requested
  int disjoint;                  // no type in two environment sets of one centre type
  const int8_t* setidx;          // [nC][256] set of a type (disjoint sets), -1 = none
  int nkI;
  uint32_t flags;
  unsigned long long* rdf_core;  // [nreal][nC][nE][H]
  unsigned long long* knn_core;  // [nreal][nC][nS][nkI][H]
  unsigned long long* counters;  // [nreal][2] pairs, centres
  uint32_t tile;                 // centres per work item
  uint32_t* work;
  int* status;
};

// ---- merged pass of several queries on one cloud (the serving loop's
// continuous batching).  Each query has its own radius, histogram geometry,
// hull-distance test, kNN orders and tasks; one walk per centre at the
// largest radius among the queries the centre belongs to serves them all.
constexpr int kMultiMaxQueries = 32;  // queries per merged pass (bits of a uint32)
constexpr int kMultiMaxTasks = 64;    // tasks per merged pass (bits of a uint64)
constexpr int kMultiMaxK = 32;        // largest kNN order (one list row per warp lane)

struct MultiQuery {
  float R, R2, Rm2;          // SpatStatRadiusMax, float(R * R), (R + grid margin)^2
  int H;                     // nbins + 2
  int cat_miss;              // category of float(R + EPSILON)
  int lut_n, lut_shift;
  uint32_t lut_base;
  uint32_t T_off, lut_off;   // offsets of its threshold table and category lookup
  uint32_t kv_off;           // offset of its kNN orders (sorted, unique, 1-based)
  int nkI, kmax;
};

struct MultiTask {
  int q;                     // its query
  uint32_t rdf;              // offset of its RDF core [H] (0xffffffff: none)
  uint32_t knn;              // offset of its kNN core [nkI][H] (0xffffffff: none)
};

struct MultiArgs {
  ScanArgs s;                          // cloud, grid, labels, row table, status
  const uint32_t* cmask;               // [n] by slot: bit q = passes query q's hull-distance test
  const uint32_t* centres;             // slots of the centres (cell order)
  uint32_t ncentres;
  int nq, nt;
  const MultiQuery* qs;                // [nq]
  const MultiTask* ts;                 // [nt]
  const uint32_t* q_of_type;           // [256] queries with a task whose targets hold the type
  const unsigned long long* t_of_type;   // [256] tasks whose targets hold the type
  const unsigned long long* env_of_type; // [256] tasks whose environment holds the type
  const unsigned long long* t_of_q;      // [nq] tasks of each query
  unsigned long long rdf_tasks, knn_tasks;  // tasks with an RDF / a kNN core
  const float* T;                      // threshold tables, all queries
  const uint16_t* lut;                 // category lookups, all queries
  const int* kvals;                    // kNN orders, all queries
  unsigned long long* rdf_core;        // flat, offsets MultiTask::rdf
  unsigned long long* knn_core;        // flat, offsets MultiTask::knn
  unsigned long long* counters;        // [nq][2] pairs, centres
  uint32_t rdf_words;                  // RDF counters of all tasks (binned in shared memory when > 0)
  int lists;                           // most kNN tasks of one centre type: list rows per warp
  uint32_t tile;                       // centres per block work item
  uint32_t* work;
};

// kernel launchers (pp_kernels.cu)
void launch_bbox(const float* xyz, uint64_t n, float* d_minmax, cudaStream_t s);
void launch_bbox_pos(const uint32_t* be, uint64_t n, float* d_minmax, cudaStream_t s);
void launch_decode_pos(const uint32_t* be, uint64_t n, const float* lo, const float* hi,
                       const uint8_t* type, int nranges, float* xyz, uint8_t* label, cudaStream_t s);
void launch_cell_count(const float* xyz, uint64_t n, Grid g, uint32_t* cell_of, uint32_t* rank,
                       uint32_t* counts, cudaStream_t s);
void launch_exclusive_scan_u32(uint32_t* data, uint64_t n, uint32_t* tmp, uint64_t tmp_elems,
                               cudaStream_t s);
void launch_scatter(const float* xyz, const uint8_t* label, uint64_t n, const uint32_t* cell_of,
                    const uint32_t* rank, const uint32_t* cell_start, float4* ions,
                    uint32_t* slot_of_id, uint32_t* id_of_slot, uint8_t* label_sorted,
                    cudaStream_t s);
void launch_gather_labels(const uint8_t* src_by_id, const uint32_t* id_of_slot, uint64_t n,
                          uint8_t* dst_by_slot, int nsets, cudaStream_t s);
void launch_permute_labels(const uint8_t* label_by_id, const uint32_t* perm, const uint32_t* id_of_slot,
                           uint64_t n, uint8_t* dst_by_slot, cudaStream_t s);
void launch_surface_cells(const float4* ions, const uint32_t* cell_start, Grid g, int f, const float* tri_box,
                          const float* tri, const uint32_t* tcs, const uint32_t* tct, Grid tg, float rprime,
                          float* surf, cudaStream_t s);
// packed caller-order xyz in, ion2surf out in the same order (no cell sort)
void launch_surface_xyz(const float* xyz, uint64_t n, const float* tbox, const float* tri, const uint32_t* tstart,
                        const uint32_t* tlist, Grid tg, float rp, float* out, cudaStream_t s);
void launch_tri_box(const float* tri, uint64_t ntri, float* box, cudaStream_t s);
// ions per voxel of the occupancy grid (lo = grid origin, nv = voxels per axis)
void launch_voxel_count(const float* xyz, uint64_t n, const float* lo, float w, const uint32_t* nv, uint32_t* occ,
                        int* status, cudaStream_t s);
// adds the list entries binning into tg makes to *total (caller zeroes it)
void launch_tri_entries(const float* tbox, uint64_t ntri, Grid tg, float grow, unsigned long long* total,
                        cudaStream_t s);
// Order-preserving centre compaction; flags needs n + 1 words, scan_tmp the
// exclusive-scan scratch for n + 1 elements.
void launch_select_centres(const uint8_t* labels, const float* surf_d2, uint64_t n, float R2,
                           const int8_t* cslot_of, const uint8_t* extra_mask, uint32_t* flags,
                           uint32_t* scan_tmp, uint64_t scan_tmp_elems, uint32_t* out,
                           uint32_t* count, uint8_t* cflag, cudaStream_t s);
// Exclusive prefix over cells of the non-centre ion count (ncells + 1 words).
void launch_nc_prefix(const uint32_t* cell_start, uint64_t ncells, const uint8_t* cflag, uint32_t* out,
                      uint32_t* scan_tmp, uint64_t scan_tmp_elems, cudaStream_t s);
// (dy, dz) stencil row offsets, [ROW_TABLE_ENTRIES][2], for ScanArgs::rowtab
const int8_t* row_table_host(int* entries);
// Bin triangles (boxes tbox[6 t]) into every cell of tg their box grown by
// rp + slack reaches; fills tstart (ncells + 1) and tlist (returns the count).
int launch_tri_bins(const float* tbox, uint64_t ntri, Grid tg, float grow, uint32_t* tstart, uint32_t* tfill,
                    uint32_t* tlist, uint64_t list_cap, uint32_t* scan_tmp, uint64_t scan_tmp_elems,
                    uint64_t* total_out, cudaStream_t s);
int launch_scan(const ScanArgs& a, int kr, int emax, int sm_count, size_t* smem_used, cudaStream_t s);
// the brick variant of k_scan; -3 when it does not apply to these arguments
int launch_brick(const ScanArgs& a, int kr, int sm_count, size_t* smem_used, cudaStream_t s);
// centre-per-lane brick scan of RDF / RIPK passes (k_lanes); -3 = not applicable
int launch_lanes(const ScanArgs& a, int kr, int sm_count, size_t* smem_used, cudaStream_t s);
// *out += the number of non-empty cells (cell_start has ncells + 1 entries)
void launch_count_occupied(const uint32_t* cell_start, uint64_t ncells, unsigned long long* out, int sm_count,
                           cudaStream_t s);
// centre-per-lane block scan of kNN-only passes (k_lanes_knn); disjoint_sets:
// every type in at most one environment set of each centre type
// (ScanArgs::setidx valid); -3 = not applicable
int launch_lanes_knn(const ScanArgs& a, bool disjoint_sets, int sm_count, size_t* smem_used, cudaStream_t s);
int launch_apply(const ApplyArgs& a, int sm_count, cudaStream_t s);
// Batched kNN in two phases, 32 realisations per warp (one per lane).
// Walk: per (centre, realisation) the category of the k-th member of every
// environment set, as records rec[centre][slot][32] (slot = set * nkI + order,
// 0xffff = no such slot) and rec_c[centre][32] (centre type slot, 0xff = not a
// centre).  Bin: per (slot, centre range) a shared [nC][H][32] histogram.
struct KnnArgs {
  const uint32_t* centres;          // geometry centres (sorted slots)
  uint32_t ncentres;                // all geometry centres
  uint32_t c0, cn;                  // centres of this launch: [c0, c0 + cn)
  const unsigned long long* pair_off;
  const uint32_t* pair_slot;
  const uint16_t* pair_cat;
  unsigned long long pair_base;     // pair_slot/pair_cat hold list positions from pair_base on
  const uint8_t* labels;            // [ngroups][n][32]
  const uint8_t* centre_ok;         // [ngroups][ncentres][32]
  uint64_t n;
  int grp, nreal;
  const int8_t* cslot_of;
  const uint32_t* envbits;          // [nC][256]
  int disjoint;                     // no type in two sets of one centre type
  const int8_t* setidx;             // [nC][256] set of a type when disjoint, -1 = none
  const int* nsets;                 // [nC]
  const int* set_list;              // [nC][32]
  const int* kvals;
  int nkI, kmax, nsmax, nC, nS, H, cat_miss;
  uint16_t* rec;                    // [cn][nsmax * nkI][32]
  uint8_t* rec_c;                   // [cn][32]
  uint32_t* work;
  uint32_t tile;                    // centres per walk work item / per bin work item
  int cblk;                         // centre types per bin histogram (set by knn32_check)
  unsigned long long* knn_core;     // [nreal][nC][nS][nkI][H]
};
// -2 when a warp's records or the bin histogram do not fit shared memory
int knn32_check(KnnArgs& k);
int launch_knn_walk(const KnnArgs& k, int sm_count, cudaStream_t s);
int launch_knn_bin(const KnnArgs& k, int sm_count, cudaStream_t s);

// n-point correlations (AnalysisSpatDistrType 5): per centre and task, the
// K-th nearest environment member's difference vector binned in a cubic grid
struct NpcArgs {
  const uint32_t* id_of_slot;       // ties in distance go to the lower ion id
  int K;                            // SpatStatKNNOrder + 1 (<= 32)
  const int* ntk;                   // [nC] tasks whose targets hold the centre type
  const int* tk_task;               // [nC][32] those tasks
  const int* tk_set;                // [nC][32] their environment set (local index)
  int half;                         // histogram half edge (voxels)
  uint32_t edge;                    // 1 + 2 half
  float inv_w;                      // 1 / SpatStatRadiusIncr (float)
  float rmax;                       // SpatStatRadiusMax: longer vectors are not binned
  uint32_t* counts;                 // [ntasks][edge^3]
};
int launch_npcorr(const ScanArgs& a, const NpcArgs& p, int sm_count, cudaStream_t s);
// guard zone of the clustered slots (clus != 0), then, in the same array, the
// labels of the statistics after clustering: 1 free, 2 guard, 3 clustered
void launch_guard(const ScanArgs& a, const uint8_t* clus, uint8_t* guard_then_labels, uint64_t n, int sm_count,
                  cudaStream_t s);

// merged multi-query pass: hull-distance bits, centre selection, the scan
void launch_cmask_or(const float* surf, uint64_t n, const float* R2, const uint32_t* bits, int nb, uint32_t* cmask,
                     cudaStream_t s);
void launch_multi_select(const uint8_t* labels, const uint32_t* cmask, const uint32_t* q_of_type, uint64_t n,
                         uint32_t* flags, uint32_t* scan_tmp, uint64_t scan_tmp_elems, uint32_t* out, uint32_t* count,
                         cudaStream_t s);
int launch_multi(const MultiArgs& m, int sm_count, size_t* smem_used, cudaStream_t s);

// neighbours within R of every slot (j != i), written by input index
void launch_ball_count(const ScanArgs& a, const uint32_t* id_of_slot, uint64_t n, uint32_t* count_by_id, int sm_count,
                       cudaStream_t s);

constexpr int kApplyThreads = 1024;
// picks the realisation group and where kNN bins accumulate; -2 = no fit
int apply_configure(ApplyArgs& a);
void launch_max_u32(const uint32_t* v, uint64_t n, uint32_t* out, cudaStream_t s);
void launch_interleave(const uint8_t* src, uint64_t rows, uint64_t cols, int G, uint8_t* dst, cudaStream_t s);
void launch_roi_mask(const float4* ions, const uint32_t* centres, uint32_t ncentres, const float* rois,
                     int nrois, float R, const uint8_t* labels, const int8_t* cslot_of,
                     uint8_t* centre_ok, cudaStream_t s);
void launch_perm_mask(const uint8_t* labels_r, const uint32_t* centres, uint32_t ncentres,
                      const int8_t* cslot_of, uint8_t* centre_ok, cudaStream_t s);
void launch_exclusive_scan_u64_from_u32(const uint32_t* in, uint64_t n, unsigned long long* out,
                                        unsigned long long* tmp, uint64_t tmp_elems, cudaStream_t s);
void launch_neighbors(const float4* ions, const uint32_t* cell_start, Grid g, uint32_t self,
                      float R, const uint32_t* id_of_slot, uint32_t* out_slot, float* out_d2,
                      uint32_t cap, uint32_t* count, cudaStream_t s);

unsigned long long kernel_launches();
// FP64 audit of the float distances and bins of the selected centres.
void launch_audit(const ScanArgs& a, double start, double scale, double end, double R64, int nbins, uint32_t stride,
                  unsigned long long* out, uint32_t* list_slots, double* list_d, uint32_t cap, int sm_count,
                  cudaStream_t s);

}  // namespace pp
