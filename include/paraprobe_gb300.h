/*
 * paraprobe_gb300.h -- C ABI of the GB300 spatial-statistics path.
 *
 * Replaces, as a drop-in boundary, the in-process call the reference makes at
 *   solver::characterize_spatstat -> horderdist::compute_generic_spatstat3
 *   (src/PARAPROBE_SolverHdl.cpp:745-776, :3685-4297)
 * together with the inputs that call reads: the ion positions and labels
 * (threadmemory::ionpp3_kdtree, src/PARAPROBE_SolverHdl.h:133), the squared
 * ion-to-hull distances (ion2surf_kdtree, :134; computed by
 * solver::surface_distancing2, src/PARAPROBE_SolverHdl.cpp:312-479), the task
 * list (horderdist::spatstat_tasks, src/PARAPROBE_SolverHdl.h:322, parsed by
 * parse_tasks, src/PARAPROBE_PeriodicTable.cpp:653-690) and the Settings
 * statics SpatStatRadiusMin/Incr/Max and SpatStatMKNNCode
 * (src/PARAPROBE_Settings.cpp:473-503).
 *
 * Conventions
 *   - Every function returns PP_OK (0) or a negative PP_ERR_* code and never
 *     aborts the process.  pp_last_error() describes the last failure.
 *   - The caller owns every host array; the library copies inputs and never
 *     keeps a host pointer.  The library owns all device memory.
 *   - One context per host thread; calls on one context are not re-entrant.
 *   - pp_run* enqueue work on the caller's CUDA stream (NULL = the legacy
 *     default stream) and return; pp_fetch* synchronise that stream.
 *   - Results are exact uint64 counts.  The reference holds the same counts
 *     as integral doubles; the CSV writer converts them when printing.
 *   - Histogram layout: one histogram is H = nbins + 2 counts
 *       [lowest, bin 0, ..., bin nbins-1, highest]
 *     with nbins = (size_t)((rmax - rmin) / rincr) evaluated in double from
 *     the float settings (src/PARAPROBE_Histogram.h:53-93).  pp_fetch writes
 *     the groups RDF[ntasks], 1NN[ntasks], RIPK[ntasks], MKNN[ntasks][nk], in
 *     that order, each present only when its flag was given to pp_run.
 *   - Type masks: 8 uint32 words per task, bit t of word t/32 set when ion
 *     type id t (0 = Unknown, ids as assigned by ranging) is in the set.
 */
#ifndef PARAPROBE_GB300_H
#define PARAPROBE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* error codes */
#define PP_OK 0
#define PP_ERR_INVALID (-1)     /* bad argument or inconsistent sizes */
#define PP_ERR_CUDA (-2)        /* a CUDA call failed */
#define PP_ERR_NOMEM (-3)       /* device or host allocation refused */
#define PP_ERR_UNSUPPORTED (-4) /* a feature outside this build's limits */
#define PP_ERR_STATE (-5)       /* call order violated (e.g. run before tasks) */
#define PP_ERR_OVERFLOW (-6)    /* a device capacity was exceeded */
#define PP_ERR_DEVICE (-7)      /* a kernel reported a failure in its status word */
#define PP_ERR_IO (-8)          /* a file could not be read or written */

/* analysis flags: the digits of AnalysisSpatDistrType
 * (src/PARAPROBE_Settings.cpp:348-392) as bits */
#define PP_RDF 1u
#define PP_1NN 2u
#define PP_RIPK 4u
#define PP_MKNN 8u
#define PP_NPCORR 16u /* n-point correlations (pp_run only; order via option "npcorr_order") */
#define PP_CNTNB 32u

#define PP_TYPE_WORDS 8 /* 256 ion types */
#define PP_TILE_LANES 0x100u /* tile code (b << 16) | PP_TILE_LANES: see pp_cloud_tuning */

typedef struct pp_ctx pp_ctx;

/* Context on CUDA device `device`.  Replaces the OpenMP team the reference
 * opens inside compute_generic_spatstat3 (src/PARAPROBE_SolverHdl.cpp:3770). */
int pp_create(pp_ctx** out, int device);
void pp_destroy(pp_ctx* ctx);
const char* pp_strerror(int code);
const char* pp_last_error(pp_ctx* ctx);

/* Upload one labelled ion cloud (host arrays): xyz is n x 3 float32,
 * label is n type ids, ion_id (nullable) are the caller's ids reported by
 * pp_neighbors (default: the input index).  Replaces the per-thread copies
 * threadmemory::read_localions builds (src/PARAPROBE_SolverHdl.cpp:1330-1468)
 * and the per-thread KD-trees of build_local_kdtree (:1593-1663): the cloud
 * is binned on the device into a uniform cell grid instead. */
int pp_cloud_upload(pp_ctx* ctx, const float* xyz, const uint8_t* label,
                    const uint32_t* ion_id, uint64_t n, int* cloud);
/* Same, from device-resident arrays (no host copy); runs on `stream`. */
int pp_cloud_upload_device(pp_ctx* ctx, const float* d_xyz, const uint8_t* d_label,
                           uint64_t n, int* cloud, void* stream);
/* Ingest a raw POS byte image (n records of big-endian float32 x, y, z, m/q,
 * src/PARAPROBE_EPOSEndianness.h:40-79) and range it on the device: the first
 * range [lo, hi] (inclusive) containing m/q gives the type, else 0
 * (PeriodicTable::mq2ionname, src/PARAPROBE_PeriodicTable.cpp:65-91).
 * Ranges must be listed in the order mq2ionname visits them. */
int pp_cloud_upload_pos(pp_ctx* ctx, const void* pos_bytes, uint64_t n,
                        const float* range_lo, const float* range_hi,
                        const uint8_t* range_type, int nranges, int* cloud);
/* Release a cloud.  The context keeps the device buffers of up to two freed
 * clouds and gives them to later uploads (no cudaMalloc / cudaFree in an
 * upload-run-free loop); pp_destroy releases them. */
int pp_cloud_free(pp_ctx* ctx, int cloud);
/* Type ids of a cloud in input order (n bytes), e.g. after pp_cloud_upload_pos. */
int pp_cloud_labels(pp_ctx* ctx, int cloud, uint8_t* label_out, uint64_t n);

/* Attach a closed triangle hull (ntri x 9 float32: v1, v2, v3) to a cloud.
 * pp_run then computes ion2surf with R' = max(rmax, carve_radius) exactly as
 * solver::surface_distancing2 does (src/PARAPROBE_SolverHdl.cpp:312-479). */
int pp_hull_upload(pp_ctx* ctx, int cloud, const float* tri, uint64_t ntri,
                   float carve_radius);
/* Or give precomputed squared distances (n floats, input order). */
int pp_surfdist_upload(pp_ctx* ctx, int cloud, const float* d2);
/* The ion2surf values pp_run used last for this cloud (n floats, input order). */
int pp_surfdist_fetch(pp_ctx* ctx, int cloud, float* d2_out, uint64_t n);

/* NumberOfIonsInside and VolumeInside, the two values heading the RDF reports:
 * the occupancy grid of vxlizer::rectangular_binning
 * (src/PARAPROBE_SolverHdl.cpp:5342-5386) with voxel edge 0.5 (bin_width_min +
 * bin_width_max) (Settings AdvIonPruneBinWidthMin/Max), its Hoshen-Kopelman
 * vacuum, surface and inside voxels (:5059-5270,
 * src/PARAPROBE_HoshenKopelman.cpp).  voxels (nullable) receives 6 counts:
 * vacuum, surface and inside voxels, then nx, ny, nz. */
int pp_cloud_inside(pp_ctx* ctx, int cloud, float bin_width_min, float bin_width_max, uint64_t* nions_inside,
                    float* volume_inside, uint64_t* voxels);

/* ion2surf without any device allocation, for callers that cannot call
 * cudaMalloc (a host whose own pool owns the device memory, a loop that may
 * not take the synchronisation cudaFree implies).  No counterpart in the
 * reference.  All pointers are device memory of the current device: xyz holds
 * n packed (x, y, z) floats, tri ntri triangles of 9 floats, d2_out receives n
 * floats in input order -- the same values pp_hull_upload + pp_run +
 * pp_surfdist_fetch give for R' = max(rmax, carve radius).  The triangle
 * boxes, grid and lists live in one static 64 MiB array per device, held until
 * exit; hulls above 2,000,000 triangles are rejected with PP_ERR_UNSUPPORTED,
 * hulls whose lists still do not fit with PP_ERR_OVERFLOW.  The first call on
 * a device looks the array up (cudaGetSymbolAddress); with the runtime's lazy
 * module loading (the default) that is when the 64 MiB are taken, so a caller
 * whose own pool takes the whole device first makes one call with n = 0 (set-up
 * only, no other argument is read but rp) on each device, before the pool
 * takes it and before any stream capture.  The address is cached per device:
 * not usable across cudaDeviceReset.  Calls share the array: calls whose GPU
 * work overlaps (different streams, unordered threads) race.  A message goes
 * to err (err_cap bytes) when it is not NULL.  stream may be NULL. */
int pp_surfdist_noalloc(const float* xyz, uint64_t n, const float* tri, uint64_t ntri, float rp,
                        float* d2_out, void* stream, char* err, size_t err_cap);

/* Task list: ntasks x PP_TYPE_WORDS words each for the centre (trg) and the
 * environment (env) sets of TypeSpecDescrStat
 * (src/PARAPROBE_PeriodicTable.h:100-128). */
int pp_tasks_set(pp_ctx* ctx, const uint32_t* trg_mask, const uint32_t* env_mask,
                 int ntasks);
/* SpatStatRadiusMin / Incr / Max as the reference stores them (float). */
int pp_hist_params(pp_ctx* ctx, float rmin, float rincr, float rmax);

/* One pass of compute_generic_spatstat3 over a cloud.  flags: PP_RDF |
 * PP_1NN | PP_RIPK | PP_MKNN | PP_CNTNB.  k_list: the MKNN orders (1-based),
 * in output order (the reference sorts them descending,
 * src/PARAPROBE_SolverHdl.cpp:3739-3763).  label_perm (nullable, n entries):
 * ion i takes the label of ion label_perm[i] for this run (the label-shuffle
 * null model of rndlabeler, src/PARAPROBE_SolverHdl.cpp:2809-3003). */
int pp_run(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk,
           const uint32_t* label_perm, void* stream);
/* pp_run with the centres restricted further: centre_mask holds n bytes in
 * input order (host memory), and only ions whose byte is nonzero may be
 * centres, on top of the reference's filter (type is a target, ion2surf >=
 * R^2, src/PARAPROBE_SolverHdl.cpp:3847-3859).  Neighbours stay every ion.
 * Used to sample centres (the results equal the reference's per-centre loop
 * run over those centres only) and for caller-defined regions.  The
 * reference has no such mask; its per-centre loop is the same. */
int pp_run_masked(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk,
                  const uint32_t* label_perm, const uint8_t* centre_mask, void* stream);
/* Descriptive statistics after clustering, for the current histogram
 * settings and hull (clustertask::flag2exclude_guard and generic_spatstat,
 * src/PARAPROBE_SolverHdl.cpp:4790-4945).  clustered: n bytes in input order,
 * nonzero = the ion belongs to a cluster.  Guard zone: every unclustered ion
 * within R (float d^2 <= R^2) of a clustered ion.  Centres: unclustered,
 * unguarded ions at least R from the hull; their neighbours: every unclustered
 * ion within R, of any type.  flags: PP_RDF and PP_RIPK count every
 * neighbour, PP_1NN the closest (a centre without one adds nothing).  The
 * result is one task in the pp_fetch layout; the tasks set with pp_tasks_set
 * stay as they were.  The reference's guard loop flags ions_kdtree.at(cand),
 * the candidate's position in its result list, instead of the candidate
 * itself (:4807-4815); by default this library flags the candidate.  With
 * option "aposteriori_guard" = 1 it runs the loop as the reference does
 * instead, positions being the cloud's input order (upload the ions in the
 * order of the clustering task's KD-tree, ions_kdtree, :4737-4787): for each
 * position i in order whose ion is clustered -- flagged, or relabelled by an
 * earlier step -- the ions at positions 0 .. |ball(i)| - 1 take i's clustered
 * type (flag_as_guarded returns a clustered type unchanged, :4576-4582), so
 * they leave the statistics as centres and as neighbours. */
int pp_run_aposteriori(pp_ctx* ctx, int cloud, const uint8_t* clustered, uint32_t flags, void* stream);
/* Project-written autotuner: times the pass on about `sample` centres
 * (0 = 200000; at least 8192 per SM, so that every kernel form fills the GPU)
 * for cell edges R/2 .. R/5 -- for passes the centre-per-lane
 * scan takes, at the default cell block of that edge (about a warp of
 * centres) and two fixed shapes; for other passes with the per-centre scan at
 * block tiles of 32, 128 and 512 centres and with the brick scan at bricks of
 * 4, 8 and 16 cells, and for passes with RDF / RIPK and kNN together (no
 * CNTNB or NPCORR) of dense centres also as two centre-per-lane passes at
 * those cell blocks -- keeps the fastest for this
 * cloud and rebuilds its cell grid.  best_tile comes back in the
 * pp_cloud_tuning encoding.  Uses the current tasks and histogram settings;
 * results of the trial runs are discarded.  Has no counterpart in the
 * reference (its KD-tree has no tuning). */
int pp_autotune(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk,
                uint32_t sample, float* best_ratio, uint32_t* best_tile);
/* Set the tuning of a cloud directly: cell edge R / cell_ratio, and a tile
 * code: 1..65535 = the per-centre scan with that many centres per block work
 * item; (b << 16) | c with b in 1..64 and c in 1..32 = the brick scan, a warp
 * taking up to c centres of b consecutive cells of a grid row together (used
 * for passes without CNTNB whose kNN, if any, has k <= 32 and disjoint
 * environment sets; other passes use the per-centre scan);
 * ((bx | by << 8 | bz << 12) << 16) | PP_TILE_LANES with bx in 1..64 and by,
 * bz in 0..15 (0 = 1) = blocks of bx x by x bz cells for the centre-per-lane
 * scan that RDF / RIPK passes without CNTNB take (one centre per lane, the
 * block's stencil ions staged in shared memory; default 4 x 2 x 2), leaving
 * the other code as it was.  With a cell block set this way, a pass with
 * RDF / RIPK and kNN together (no CNTNB or NPCORR) runs as two passes: the
 * RDF / RIPK part on the centre-per-lane scan, then the kNN part on the
 * centre-per-lane kNN scan (the per-centre scan for overlapping environment
 * sets or lists too large for shared memory).  Results do not depend on the
 * tuning. */
int pp_cloud_tuning(pp_ctx* ctx, int cloud, float cell_ratio, uint32_t tile);

/* FP64 audit of the current tasks and histogram settings on up to
 * max_centres centres (evenly spaced over the cell-ordered centre list; 0 =
 * all): every candidate within R is recomputed in double precision from the
 * same float coordinates.  Reports the largest absolute and relative error of
 * the float distance, the number of pairs audited, the pairs whose float bin
 * (the reference's arithmetic) differs from the exact double bin, and the pairs
 * on which float and double disagree about d <= R; up to `cap` disagreements
 * are listed as (centre id, neighbour id) with (d_float, d_double).  A
 * diagnostic with no counterpart in the reference. */
int pp_fp64_audit(pp_ctx* ctx, int cloud, uint32_t max_centres, double* max_abs, double* max_rel,
                  uint64_t* pairs, uint64_t* bin_disagree, uint64_t* set_disagree,
                  uint64_t* listing_ids, double* listing_d, uint64_t cap, uint64_t* nlisted);

/* n-point correlations of the last pp_run with PP_NPCORR
 * (src/PARAPROBE_SolverHdl.cpp:3899-3955, src/PARAPROBE_NPointCorrelations3D.cpp):
 * per task a cubic histogram of edge = 1 + 2 (ceil(rmax / rincr) + 1) voxels
 * a side, counts[task][z][y][x], of the difference vector (neighbour minus
 * centre) of each centre's (order+1)-th nearest environment member within
 * rmax, order = option "npcorr_order" (SpatStatKNNOrder - 1, default 0).
 * Exact distance ties go to the lower ion id.  Histograms above 503^3 voxels
 * are refused with PP_ERR_UNSUPPORTED, as the reference refuses them.  With
 * counts == NULL only *edge is set. */
int pp_fetch_npcorr(pp_ctx* ctx, uint32_t* counts, uint64_t cap, uint64_t* edge);

/* Context options:
 *   "symmetric"         RDF/RIPK-only passes take each pair of two centres
 *                       once and credit both (default 1); 0 scans every
 *                       centre's full ball.  Results are identical either way.
 *   "lanes"             RDF/RIPK-only passes take the centre-per-lane brick
 *                       scan (default 1); 0 = the per-centre or brick scan.
 *                       Results are identical either way.
 *   "uniform_sets"      the kNN centre-per-lane scan stages one set row per ion
 *                       when every centre type maps types to sets alike
 *                       (default 1); 0 decodes the set per centre slot.
 *                       Results are identical either way.
 *   "knn_lists"         lists of the kNN centre-per-lane scan: 0 = distances
 *                       while they fit two blocks per SM, bin categories
 *                       beyond (default); 1 = distances; 2 = categories.
 *                       Results are identical either way.
 *   "box_filter"        the centre-per-lane scans test only ions within R of
 *                       the bounding box of a batch's centres (default 1);
 *                       0 tests every ion of the block's stencil rows.
 *                       Results are identical either way.
 *   "npcorr_order"      SpatStatKNNOrder - 1 for PP_NPCORR (0..31, default 0).
 *   "server_batch"      most queries per merged serving pass (1..32, default
 *                       32; 1 = every query alone), read by pp_server_create.
 *   "aposteriori_guard" pp_run_aposteriori's guard zone: 0 = every
 *                       unclustered ion within R of a clustered ion (default),
 *                       1 = the reference's guard loop as written (see there).
 *   "batched_pair_cap"  most pairs pp_run_batched holds at once; larger lists
 *                       are built and applied a chunk of centres at a time
 *                       (0 = sized from free device memory, the default). */
int pp_set_option(pp_ctx* ctx, const char* name, int value);

/* Results of the last pp_run (synchronises). cap = capacity in uint64. */
int pp_fetch(pp_ctx* ctx, uint64_t* bins, size_t cap);
/* Neighbour-count histograms (PP_CNTNB): ntasks x len counts; *len returns
 * the common length (largest count + 1).  Pass bins = NULL to query *len. */
int pp_fetch_cntnb(pp_ctx* ctx, uint64_t* bins, size_t cap, uint64_t* len);
/* Number of uint64 pp_fetch writes and the bin count per histogram. */
int pp_result_size(pp_ctx* ctx, uint64_t* total, uint64_t* nbins);
/* Centres considered, ions discarded, and in-ball (centre, neighbour) pairs
 * of the last run (the considered/discarded counts printed at
 * src/PARAPROBE_SolverHdl.cpp:4112-4116). */
int pp_run_stats(pp_ctx* ctx, uint64_t* centres, uint64_t* discarded, uint64_t* pairs);

/* Batched realisations in one persistent launch: the plain labels
 * (include_original != 0), then n_label_sets label arrays (n_label_sets x n
 * type ids, input order, host or device memory), then n_rois spherical
 * regions of interest (n_rois x 4 float: cx, cy, cz, radius; a centre must
 * satisfy radius - |p - c| >= rmax in addition to the plain filter, the
 * environment stays the whole cloud).  Same flags and k_list as pp_run. */
int pp_run_batched(pp_ctx* ctx, int cloud, uint32_t flags, const uint32_t* k_list, int nk,
                   int include_original, const uint8_t* label_sets, int n_label_sets,
                   const float* rois, int n_rois, void* stream);
/* Number of realisations of the last batched run. */
int pp_batched_count(pp_ctx* ctx, int* n_realisations);
/* Results of realisation r of the last batched run, pp_fetch layout. */
int pp_fetch_batched(pp_ctx* ctx, int r, uint64_t* bins, size_t cap);
int pp_batched_stats(pp_ctx* ctx, int r, uint64_t* centres, uint64_t* pairs);
/* The device work of a batched run (the realisation passes after the pair
 * lists and label layouts are built) runs as one CUDA graph: captured when
 * its launch parameters change, replayed otherwise.  Nodes of the current
 * graph, captures and launches so far.  No counterpart in the reference. */
int pp_batched_graph(pp_ctx* ctx, uint64_t* nodes, uint64_t* captures, uint64_t* launches);

/* Neighbour set of one ion (input index): every other ion with float
 * d^2 <= r^2, d^2 = (xi-xj)^2 + (yi-yj)^2 + (zi-zj)^2 evaluated left to right
 * without contraction (src/PARAPROBE_KDTree.h:55-58), sorted by (d^2, id). */
int pp_neighbors(pp_ctx* ctx, int cloud, uint64_t ion, float r, uint64_t* ids,
                 float* d2, uint64_t cap, uint64_t* count);

/* Deterministic label shuffle for the null model: a Fisher-Yates pass driven
 * by splitmix64(seed).  The reference's std::shuffle over mt19937 is
 * implementation-defined and depends on its thread count, so both sides of a
 * comparison take the permuted labels this produces. */
int pp_shuffle_labels(const uint8_t* label, uint64_t n, uint64_t seed, uint8_t* out);

/* Number of kernels this library has launched in the process so far. */
int pp_kernel_launches(uint64_t* count);
/* Device time of the last run's main kernel (the stencil scan of pp_run, the
 * realisation pass of pp_run_batched), measured with CUDA events recorded
 * around that launch on the run's stream.  Synchronises. */
int pp_last_kernel_ms(pp_ctx* ctx, float* ms);
/* Name of the stencil kernel the last pp_run took: "k_scan" (per-centre
 * scan), "k_brick" (brick scan), "k_lanes" (centre-per-lane scan of RDF /
 * RIPK passes) or "k_lanes_knn" (centre-per-lane scan of kNN passes); a static
 * string; "k_lanes+k_lanes_knn" or "k_lanes+k_scan" for a pass with RDF /
 * RIPK and kNN run as two passes (see pp_cloud_tuning).  The centre-per-lane
 * scans take passes of dense centres (at least 0.35 per non-empty cell, or a
 * block shape set with pp_cloud_tuning) without CNTNB or NPCORR, kNN only with
 * disjoint environment sets; a pass with both RDF / RIPK and kNN takes the
 * per-centre scan unless a block shape is set.  No counterpart in the
 * reference. */
int pp_last_kernel(pp_ctx* ctx, const char** name);
/* Candidate distance tests (centre, candidate) the last pp_run evaluated --
 * an implementation figure beside the in-ball pairs of pp_run_stats (their
 * ratio is the tests per pair the cell grid and the kernel cost).  Synchronises.
 * No counterpart in the reference. */
int pp_run_tests(pp_ctx* ctx, uint64_t* tests);

/* Prepare a cloud for queries with r_lo <= rmax <= r_hi (r_hi <= 6 r_lo):
 * builds its cell grid with edge r_lo, the hull lists for R' up to
 * max(r_hi, carve radius) and the cached ion2surf for R' = max(r_lo, carve);
 * unless the cloud was tuned, passes of dense centres then take the
 * centre-per-lane scans at a 4 x 2 x 2 cell block.  Required before a cloud
 * is served. */
int pp_cloud_prepare(pp_ctx* ctx, int cloud, float r_lo, float r_hi);

/* ---- serving loop (no counterpart in the reference, which runs one task per
 * process): clouds stay resident in the context; queries are admitted by
 * estimated HBM footprint as worker slots and memory free up, and run
 * concurrently on the workers' own streams.  Continuous batching: a free
 * worker takes the oldest waiting query together with every other waiting
 * query on the same cloud (up to option "server_batch", default 32, and 64
 * tasks) and runs them as ONE merged pass -- one candidate walk per centre at
 * the largest radius among the queries the centre belongs to, each query with
 * its own radius, hull-distance test, histogram bins, tasks and kNN orders --
 * so queries that arrive while others run join the next pass on their cloud.
 * Each query's bins, pairs and centres are those pp_run gives it alone.
 * Queries whose centre types are dense (at least 0.35 target ions per
 * non-empty cell) run alone on the plain path, whose centre-per-lane scans
 * (pp_cloud_prepare sets their cell block) are faster than a shared walk for
 * them; so do queries with PP_CNTNB, PP_NPCORR or k > 32. */
typedef struct pp_server pp_server;
/* `slots` worker threads, each with its own stream and run buffers;
 * `budget_bytes` caps the estimated device memory of admitted queries. */
int pp_server_create(pp_ctx* ctx, int slots, uint64_t budget_bytes, pp_server** out);
/* Queue one query (tasks as for pp_tasks_set, histogram as for
 * pp_hist_params, flags/k_list as for pp_run).  Returns PP_ERR_NOMEM (and
 * counts a rejection) when the query could never fit the budget. */
int pp_server_submit(pp_server* srv, int cloud, uint32_t flags, float rmin, float rincr, float rmax,
                     const uint32_t* trg_mask, const uint32_t* env_mask, int ntasks,
                     const uint32_t* k_list, int nk, uint64_t* ticket);
/* Wait for a query and take its results (pp_fetch layout).  len returns the
 * number of uint64 written; latency_ms is submit-to-completion time. */
int pp_server_wait(pp_server* srv, uint64_t ticket, uint64_t* bins, size_t cap, uint64_t* len,
                   uint64_t* pairs, double* latency_ms);
/* stats[0..7]: submitted, admitted, rejected, completed, in flight,
 * p50 ms, p99 ms, total pairs of completed queries (as doubles). */
int pp_server_stats(pp_server* srv, double* stats);
/* Merged passes run so far and the queries they took. */
int pp_server_passes(pp_server* srv, uint64_t* passes, uint64_t* queries);
void pp_server_destroy(pp_server* srv);

/* Device the context runs on and its SM count. */
int pp_device_info(pp_ctx* ctx, int* device, int* sm_count);

#ifdef __cplusplus
}
#endif
#endif /* PARAPROBE_GB300_H */
