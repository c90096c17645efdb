// pp_oracle.cpp -- CPU ORACLE (test infrastructure only).
//
// This file is the checker for the GB300 spatial-statistics path, not part of
// the product.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may load it.  It restates, in plain C++/OpenMP, the reference's
// CPU algorithm for PARAPROBE's descriptive spatial statistics:
//
//   * z-slab decomposition at z-quantiles, one slab per thread
//       (src/PARAPROBE_SolverHdl.cpp:1819-1934, src/PARAPROBE_Math.cpp:52-85)
//   * one median-split KD-tree per slab, leaves of <= 256 points, cyclic x/y/z,
//     points repacked into leaf order (src/PARAPROBE_KDTree.cpp:34-133,173-192)
//   * ball queries collecting every j != i with float d^2 <= R^2
//       (src/PARAPROBE_KDTree.cpp:423-655, src/PARAPROBE_KDTree.h:55-58)
//   * the per-centre accumulation of RDF, 1NN, RIPK, CNTNB and MKNN
//       (src/PARAPROBE_SolverHdl.cpp:3685-4177)
//   * fixed-width double histograms with lowest/highest dumps
//       (src/PARAPROBE_Histogram.h:53-117)
//   * the ion-to-hull squared distance used to exclude centres near the
//     specimen surface (src/PARAPROBE_SolverHdl.cpp:312-479,
//     src/PARAPROBE_Math.cpp:88-184, src/PARAPROBE_AABBTree.cpp:112-124)
//   * the occupancy grid that gives the RDF header its NumberOfIonsInside and
//     VolumeInside (src/PARAPROBE_SolverHdl.cpp:5059-5386, 1471-1508; the
//     outer vacuum is the face-connected cluster of empty voxels holding the
//     guard corner, which src/PARAPROBE_HoshenKopelman.cpp labels)
//   * the statistics after clustering, centres outside a guard zone about the
//     clustered ions (src/PARAPROBE_SolverHdl.cpp:4790-4945)
//
// The restatement is pinned against the reference's own units compiled from
// the read-only reference tree (oracle/ref/), through golden fixtures under
// tests/golden/.  Build with -ffp-contract=off: every float expression below
// must round exactly as the reference's does, without fused multiply-adds.
//
// Output layout (shared with the CUDA library's pp_fetch):
//   H = nbins + 2 uint64 per histogram: [lowest, bin 0 .. bin nbins-1, highest]
//   groups in this order, each present only if its analysis was requested:
//     RDF  [ntasks][H], 1NN [ntasks][H], RIPK [ntasks][H], MKNN [ntasks][nk][H]
//   CNTNB is returned separately as [ntasks][cntnb_len] counts.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#include <omp.h>

namespace {

constexpr uint32_t A_RDF = 1u, A_1NN = 2u, A_RIPK = 4u, A_MKNN = 8u, A_CNTNB = 32u;
constexpr double kEpsilon = 1.0e-6;  // src/PARAPROBE_Numerics.h:44 (EPSILON)

// ---------------------------------------------------------------- histogram
// Follows src/PARAPROBE_Histogram.h:53-117: bin count (end-start)/width taken
// in double from float settings; add() maps x through double, rounds the bin
// coordinate to float, floors it, and dumps x == end (b == nbins) to highest.
struct Hist {
  double start = 0, width = 0, end = 0, scale = 0;
  uint32_t nbins = 0;
  std::vector<double> cnt;  // [lowest, bins..., highest]
  void init(float s, float w, float e) {
    start = s; width = w; end = e;
    size_t nb = 0;
    if (width > kEpsilon) nb = (size_t)((end - start) / width);
    nbins = (uint32_t)nb;
    scale = nbins ? 1.0 / (end - start) * (double)nbins : 0.0;
    cnt.assign(nbins + 2, 0.0);
  }
  inline void add(float x) {
    double xx = x;
    if (xx >= start && xx <= end) {
      float rb = (float)((xx - start) * scale);
      uint32_t b = (uint32_t)std::floor(rb);
      if (b < nbins) cnt[1 + b] += 1.0; else cnt[nbins + 1] += 1.0;
    } else {
      if (xx < start) cnt[0] += 1.0;
      if (xx > end) cnt[nbins + 1] += 1.0;
    }
  }
  void merge(const Hist& o) { for (size_t i = 0; i < cnt.size(); ++i) cnt[i] += o.cnt[i]; }
};

// ------------------------------------------------------------------ points
struct Ion { float x, y, z; uint32_t m; };   // 16 B record, like p3dm1
struct Nb { float d; uint32_t m; };

inline float sqr(float v) { return v * v; }
// (a-b)^2 summed left to right in float (src/PARAPROBE_KDTree.h:55-58).
inline float dist2(const Ion& a, const Ion& b) {
  return sqr(a.x - b.x) + sqr(a.y - b.y) + sqr(a.z - b.z);
}

// ----------------------------------------------------------------- KD-tree
struct Box { float lo[3], hi[3]; };
// Squared distance from p to a box, accumulated x, y, z, zero inside
// (src/PARAPROBE_KDTree.h:64-86).
inline float box_gap2(const Box& b, const Ion& p) {
  float r = 0.f;
  const float c[3] = {p.x, p.y, p.z};
  for (int k = 0; k < 3; ++k) {
    if (c[k] < b.lo[k]) r += sqr(b.lo[k] - c[k]);
    else if (c[k] > b.hi[k]) r += sqr(c[k] - b.hi[k]);
  }
  return r;
}

struct Node { size_t a = SIZE_MAX, b = SIZE_MAX; bool leaf = false; float split = 0.f; };

struct KdTree {
  std::vector<Node> nodes;
  Box bounds{};
  // Median split with nth_element on the cycling axis; a range of fewer than
  // 257 points becomes a leaf (src/PARAPROBE_KDTree.cpp:34-133).
  void build(const std::vector<Ion>& pts, std::vector<size_t>& perm) {
    nodes.clear(); perm.clear();
    const size_t n = pts.size();
    for (int k = 0; k < 3; ++k) { bounds.lo[k] = std::numeric_limits<float>::max(); bounds.hi[k] = std::numeric_limits<float>::lowest(); }
    if (n == 0) return;
    perm.resize(n);
    for (size_t i = 0; i < n; ++i) perm[i] = i;
    struct Task { size_t first, last, node; int dim; };
    std::vector<Task> st;
    nodes.emplace_back();
    st.push_back({0, n - 1, 0, 0});
    while (!st.empty()) {
      Task t = st.back(); st.pop_back();
      if (t.last - t.first < 256) {
        Node& nd = nodes[t.node];
        nd.leaf = true; nd.a = t.first; nd.b = t.last;
        for (size_t k = t.first; k <= t.last; ++k) {
          const Ion& p = pts[perm[k]];
          const float c[3] = {p.x, p.y, p.z};
          for (int d = 0; d < 3; ++d) {
            if (c[d] < bounds.lo[d]) bounds.lo[d] = c[d];
            if (c[d] > bounds.hi[d]) bounds.hi[d] = c[d];
          }
        }
        continue;
      }
      const size_t mid = (t.first + t.last) / 2;
      const int dim = t.dim;
      auto key = [&](size_t i) { const Ion& p = pts[i]; return dim == 0 ? p.x : (dim == 1 ? p.y : p.z); };
      std::nth_element(perm.begin() + t.first, perm.begin() + mid, perm.begin() + t.last + 1,
                       [&](size_t i1, size_t i2) { return key(i1) < key(i2); });
      const size_t left = nodes.size();
      nodes[t.node].split = key(perm[mid]);
      nodes[t.node].a = left;
      nodes[t.node].b = left + 1;
      nodes.emplace_back();
      nodes.emplace_back();
      const int nd = (dim + 1) % 3;
      st.push_back({mid + 1, t.last, left + 1, nd});
      st.push_back({t.first, mid, left, nd});
    }
  }
  // Every point of 'pts' (the tree's own, in leaf order) with float d^2 <= r2,
  // skipping index 'self' (src/PARAPROBE_KDTree.cpp:539-655 and :423-537).
  void ball(const Ion& q, size_t self, const std::vector<Ion>& pts, float r2, std::vector<Nb>& out) const {
    if (nodes.empty()) return;
    struct Visit { Box bx; size_t node; int dim; float gap; };
    Visit stack[64];
    int top = 0;
    stack[0] = {bounds, 0, 0, box_gap2(bounds, q)};
    while (top >= 0) {
      Visit v = stack[top--];
      if (v.gap > r2) continue;
      const Node& nd = nodes[v.node];
      if (nd.leaf) {
        for (size_t i = nd.a; i <= nd.b; ++i) {
          const float d = dist2(q, pts[i]);
          if (d <= r2 && i != self) out.push_back({std::sqrt(d), pts[i].m});
        }
        continue;
      }
      Box lo = v.bx, hi = v.bx;
      lo.hi[v.dim] = nd.split;
      hi.lo[v.dim] = nd.split;
      const float c = v.dim == 0 ? q.x : (v.dim == 1 ? q.y : q.z);
      const bool nearlo = c <= nd.split;
      const int ndim = (v.dim + 1) % 3;
      const Box& farb = nearlo ? hi : lo;
      stack[++top] = {farb, nearlo ? nd.b : nd.a, ndim, box_gap2(farb, q)};
      stack[++top] = {nearlo ? lo : hi, nearlo ? nd.a : nd.b, ndim, 0.f};
    }
  }
};

// ------------------------------------------------------ z-slab decomposition
// One slab per thread, split at z-quantiles of the sorted z column with
// lerp-based quantiles (src/PARAPROBE_Math.cpp:52-85); first and last slab
// padded by 1e-4 (src/PARAPROBE_SolverHdl.cpp:1890-1900).  Ions belong to a
// slab when zmi <= z < zmx.
inline float lerpf(float v0, float v1, float t) { return (1.f - t) * v0 + t * v1; }

struct Slab {
  float zmi, zmx;
  std::vector<Ion> ions;          // leaf order
  std::vector<float> surf;        // ion2surf, leaf order
  std::vector<uint8_t> mask;      // centre mask, leaf order
  std::vector<uint64_t> id;       // original index, leaf order
  KdTree tree;
};

void decompose(const float* xyz, const uint8_t* lab, const float* surf, const uint8_t* cmask,
               uint64_t n, int T, std::vector<Slab>& slabs) {
  std::vector<float> z(n);
  for (uint64_t i = 0; i < n; ++i) z[i] = xyz[3 * i + 2];
  std::sort(z.begin(), z.end());
  std::vector<float> qq;
  for (int t = 1; t < T; ++t) {
    const float q = (float)t / (float)T;
    const float poi = lerpf(-0.5f, (float)n - 0.5f, q);
    const size_t left = (size_t)std::max<int64_t>((int64_t)std::floor(poi), 0);
    const size_t right = (size_t)std::min<int64_t>((int64_t)std::ceil(poi), (int64_t)n - 1);
    qq.push_back(lerpf(z[left], z[right], poi - (float)left));
  }
  slabs.assign(T, Slab());
  for (int t = 0; t < T; ++t) {
    slabs[t].zmi = (t == 0) ? z.front() - 1.0e-4f : qq[t - 1];
    slabs[t].zmx = (t == T - 1) ? z.back() + 1.0e-4f : qq[t];
  }
#pragma omp parallel for schedule(static, 1) num_threads(T)
  for (int t = 0; t < T; ++t) {
    Slab& s = slabs[t];
    std::vector<Ion> raw;
    std::vector<uint64_t> rid;
    for (uint64_t i = 0; i < n; ++i) {
      const float zz = xyz[3 * i + 2];
      if (zz >= s.zmi && zz < s.zmx) {
        raw.push_back({xyz[3 * i], xyz[3 * i + 1], zz, (uint32_t)lab[i]});
        rid.push_back(i);
      }
    }
    std::vector<size_t> perm;
    s.tree.build(raw, perm);
    s.ions.resize(raw.size()); s.surf.resize(raw.size()); s.mask.resize(raw.size()); s.id.resize(raw.size());
    for (size_t k = 0; k < perm.size(); ++k) {
      const uint64_t g = rid[perm[k]];
      s.ions[k] = raw[perm[k]];
      s.surf[k] = surf ? surf[g] : std::numeric_limits<float>::max();
      s.mask[k] = cmask ? cmask[g] : 1;
      s.id[k] = g;
    }
  }
}

void gather(const std::vector<Slab>& slabs, int thr, size_t i, float R, float r2, std::vector<Nb>& nb) {
  const Slab& s = slabs[thr];
  const Ion& me = s.ions[i];
  s.tree.ball(me, i, s.ions, r2, nb);
  // Ions whose ball leaves the slab also query every other slab
  // (src/PARAPROBE_SolverHdl.cpp:3871-3896).
  if (!((me.z - R) > s.zmi && (me.z + R) < s.zmx)) {
    for (int o = 0; o < (int)slabs.size(); ++o)
      if (o != thr) slabs[o].tree.ball(me, SIZE_MAX, slabs[o].ions, r2, nb);
  }
}

inline bool bit(const uint32_t* m, uint32_t t) { return (m[t >> 5] >> (t & 31)) & 1u; }

// ------------------------------------------------------- hull distancing
// Squared distance from p to the closest point of triangle (v1,v2,v3), by the
// region case analysis of D. Eberly, "Distance Between Point and Triangle in
// 3D" -- the float evaluation order and clamp semantics follow
// src/PARAPROBE_Math.cpp:88-184 (including its region-6 fallback, which
// clamps -e/c), because ion exclusion must round exactly like the reference.
inline float clamp01(float x) {
  const float lo = (x < 0.f) ? 0.f : x;     // MAX(x,0) as (x<0)?0:x
  return (lo < 1.f) ? lo : 1.f;              // MIN(.,1) as (.<1)?.:1
}
float tri_dist2(const float* t, float px, float py, float pz) {
  const float e0x = t[3] - t[0], e0y = t[4] - t[1], e0z = t[5] - t[2];
  const float e1x = t[6] - t[0], e1y = t[7] - t[1], e1z = t[8] - t[2];
  const float vx = t[0] - px, vy = t[1] - py, vz = t[2] - pz;
  const float a = e0x * e0x + e0y * e0y + e0z * e0z;
  const float b = e0x * e1x + e0y * e1y + e0z * e1z;
  const float c = e1x * e1x + e1y * e1y + e1z * e1z;
  const float d = e0x * vx + e0y * vy + e0z * vz;
  const float e = e1x * vx + e1y * vy + e1z * vz;
  const float det = a * c - b * b;
  float s = b * e - c * d;
  float u = b * d - a * e;
  if (s + u < det) {
    if (s < 0.f) {
      if (u < 0.f) {
        if (d < 0.f) { s = clamp01(-d / a); u = 0.f; }
        else { s = 0.f; u = clamp01(-e / c); }
      } else { s = 0.f; u = clamp01(-e / c); }
    } else if (u < 0.f) {
      s = clamp01(-d / a); u = 0.f;
    } else {
      const float inv = 1.f / det;
      s *= inv; u *= inv;
    }
  } else {
    if (s < 0.f) {
      const float t0 = b + d, t1 = c + e;
      if (t1 > t0) {
        const float num = t1 - t0, den = a - 2.f * b + c;
        s = clamp01(num / den); u = 1.f - s;
      } else { u = clamp01(-e / c); s = 0.f; }
    } else if (u < 0.f) {
      if (a + d > b + e) {
        const float num = c + e - b - d, den = a - 2.f * b + c;
        s = clamp01(num / den); u = 1.f - s;
      } else { s = clamp01(-e / c); u = 0.f; }
    } else {
      const float num = c + e - b - d, den = a - 2.f * b + c;
      s = clamp01(num / den); u = 1.f - s;
    }
  }
  const float cx = t[0] + s * e0x + u * e1x;
  const float cy = t[1] + s * e0y + u * e1y;
  const float cz = t[2] + s * e0z + u * e1z;
  return sqr(cx - px) + sqr(cy - py) + sqr(cz - pz);
}

}  // namespace

extern "C" {

// ion2surf for every ion: R'^2 unless some triangle's float AABB overlaps the
// query box p +- R' (touching counts, src/PARAPROBE_AABBTree.cpp:112-124), in
// which case min(R'^2, min over those triangles of tri_dist2)
// (src/PARAPROBE_SolverHdl.cpp:335-348, :403-437).  Candidates are found
// through a uniform grid over triangle boxes instead of the reference's AABB
// tree; the candidate set is the same because both test the same boxes.
int ppo_surface_distance(const float* xyz, uint64_t n, const float* tri, uint64_t ntri,
                         float rprime, float* out_d2, int nthreads) {
  if (!xyz || !out_d2 || (ntri && !tri)) return -1;
  const float R = rprime, R2 = R * R;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  std::vector<float> bx(6 * ntri);
  float glo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(), std::numeric_limits<float>::max()};
  float ghi[3] = {std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest()};
  for (uint64_t t = 0; t < ntri; ++t) {
    const float* v = tri + 9 * t;
    for (int k = 0; k < 3; ++k) {
      const float lo = std::fmin(std::fmin(v[k], v[3 + k]), v[6 + k]);
      const float hi = std::fmax(std::fmax(v[k], v[3 + k]), v[6 + k]);
      bx[6 * t + k] = lo; bx[6 * t + 3 + k] = hi;
      glo[k] = std::min(glo[k], lo); ghi[k] = std::max(ghi[k], hi);
    }
  }
  // coarse grid of triangle boxes grown by R' (+1 cell of slack)
  const float h = std::max(2.f * R, 1.f);
  int dim[3];
  for (int k = 0; k < 3; ++k) {
    if (ntri == 0) { glo[k] = 0; ghi[k] = 0; }
    glo[k] -= (R + h); ghi[k] += (R + h);
    dim[k] = std::max(1, (int)std::ceil((ghi[k] - glo[k]) / h));
  }
  const size_t ncell = (size_t)dim[0] * dim[1] * dim[2];
  std::vector<std::vector<uint32_t>> cell(ntri ? ncell : 0);
  for (uint64_t t = 0; t < ntri; ++t) {
    int c0[3], c1[3];
    for (int k = 0; k < 3; ++k) {
      c0[k] = std::max(0, (int)std::floor((bx[6 * t + k] - R - glo[k]) / h) - 1);
      c1[k] = std::min(dim[k] - 1, (int)std::floor((bx[6 * t + 3 + k] + R - glo[k]) / h) + 1);
    }
    for (int z = c0[2]; z <= c1[2]; ++z)
      for (int y = c0[1]; y <= c1[1]; ++y)
        for (int x = c0[0]; x <= c1[0]; ++x)
          cell[((size_t)z * dim[1] + y) * dim[0] + x].push_back((uint32_t)t);
  }
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const float px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
    float best = R2;
    if (ntri) {
      const float q[3] = {px, py, pz};
      int c[3]; bool inside = true;
      for (int k = 0; k < 3; ++k) {
        c[k] = (int)std::floor((q[k] - glo[k]) / h);
        if (c[k] < 0 || c[k] >= dim[k]) inside = false;
      }
      if (inside) {
        const float lo[3] = {px - R, py - R, pz - R}, hi[3] = {px + R, py + R, pz + R};
        for (uint32_t t : cell[((size_t)c[2] * dim[1] + c[1]) * dim[0] + c[0]]) {
          const float* b = &bx[6 * t];
          if (b[3] < lo[0] || b[0] > hi[0] || b[4] < lo[1] || b[1] > hi[1] || b[5] < lo[2] || b[2] > hi[2]) continue;
          const float v = tri_dist2(tri + 9 * t, px, py, pz);
          if (!(v > best)) best = v;
        }
      }
    }
    out_d2[i] = best;
  }
  return 0;
}

// Full descriptive-statistics pass of src/PARAPROBE_SolverHdl.cpp:3685-4177.
//   xyz [n*3], label [n] (type ids, 0 = unknown), ion2surf [n] (squared, may be
//   NULL = no exclusion), centre_mask [n] (NULL = all ions eligible; a zero
//   removes that ion from the centre set only).
//   trg_mask / env_mask: ntasks x 8 words, bit t set when type t is listed.
//   k_list: MKNN orders (1-based) in output order.
//   stats (nullable): [0] centres, [1] discarded ions, [2] in-ball pairs,
//   [3] nanoseconds spent in decomposition + KD-tree builds (the reference's
//   Loadpartitioning / ThreadparallelKDTreeConstruct phases), [4] nanoseconds
//   in the statistics pass (DescrStatsThreadparallelCompute).
int ppo_spatstat(const float* xyz, const uint8_t* label, const float* ion2surf, uint64_t n,
                 float rmin, float rincr, float rmax, uint32_t analyses,
                 const uint32_t* k_list, int nk, int ntasks,
                 const uint32_t* trg_mask, const uint32_t* env_mask,
                 const uint8_t* centre_mask, int nthreads,
                 uint64_t* out_bins, uint64_t out_cap,
                 uint64_t* out_cntnb, uint64_t cntnb_len, uint64_t* stats) {
  if (!xyz || !label || ntasks < 0 || (ntasks && (!trg_mask || !env_mask))) return -1;
  if ((analyses & A_MKNN) && nk > 0 && !k_list) return -1;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  Hist proto; proto.init(rmin, rincr, rmax);
  const uint64_t H = proto.nbins + 2;
  const bool doR = analyses & A_RDF, do1 = analyses & A_1NN, doK = analyses & A_RIPK,
             doM = (analyses & A_MKNN) && nk > 0, doC = analyses & A_CNTNB;
  const uint64_t need = H * (uint64_t)ntasks * ((doR ? 1 : 0) + (do1 ? 1 : 0) + (doK ? 1 : 0) + (doM ? nk : 0));
  if (need > out_cap) return -2;
  if (doC && (!out_cntnb || cntnb_len == 0)) return -1;

  const float R = rmax;
  const float RSQR = R * R;
  const float missing = (float)(R + kEpsilon);  // add(R + EPSILON) takes an apt_real

  const double t_build0 = omp_get_wtime();
  std::vector<Slab> slabs;
  decompose(xyz, label, ion2surf, centre_mask, n, nthreads, slabs);
  const double t_build1 = omp_get_wtime();
  uint32_t maxtype = 0;
  for (uint64_t i = 0; i < n; ++i) maxtype = std::max<uint32_t>(maxtype, label[i]);
  for (int t = 0; t < ntasks; ++t)
    for (uint32_t ty = 0; ty < 256; ++ty)
      if (bit(trg_mask + 8 * t, ty) || bit(env_mask + 8 * t, ty)) maxtype = std::max(maxtype, ty);
  const uint32_t ntypes = maxtype + 1;

  std::vector<uint8_t> any_trg(256, 0);
  for (int t = 0; t < ntasks; ++t)
    for (uint32_t ty = 0; ty < 256; ++ty) if (bit(trg_mask + 8 * t, ty)) any_trg[ty] = 1;
  std::vector<std::vector<uint32_t>> env_types(ntasks);
  for (int t = 0; t < ntasks; ++t)
    for (uint32_t ty = 0; ty < 256; ++ty) if (bit(env_mask + 8 * t, ty)) env_types[t].push_back(ty);

  std::vector<Hist> gR, g1, gK, gM;
  std::vector<std::vector<uint64_t>> gC(doC ? ntasks : 0, std::vector<uint64_t>(cntnb_len, 0));
  auto mk = [&](std::vector<Hist>& v, int cnt) { v.assign(cnt, proto); };
  if (doR) mk(gR, ntasks);
  if (do1) mk(g1, ntasks);
  if (doK) mk(gK, ntasks);
  if (doM) mk(gM, ntasks * nk);
  uint64_t n_centre = 0, n_disc = 0, n_pairs = 0;
  int err = 0;

#pragma omp parallel num_threads(nthreads) reduction(+ : n_centre, n_disc, n_pairs)
  {
    std::vector<Hist> mR, m1, mK, mM;
    if (doR) mR.assign(ntasks, proto);
    if (do1) m1.assign(ntasks, proto);
    if (doK) mK.assign(ntasks, proto);
    if (doM) mM.assign(ntasks * nk, proto);
    std::vector<std::vector<uint64_t>> mC(doC ? ntasks : 0, std::vector<uint64_t>(cntnb_len, 0));
    std::vector<Nb> nb;
    std::vector<size_t> cs(ntypes + 1), fill(ntypes);
    std::vector<float> ordered, tmp;
    for (int thr = 0; thr < (int)slabs.size(); ++thr) {
      const Slab& s = slabs[thr];
#pragma omp for schedule(dynamic, 1) nowait
      for (int64_t ii = 0; ii < (int64_t)s.ions.size(); ++ii) {
        const size_t i = (size_t)ii;
        const Ion& me = s.ions[i];
        const bool considerme = any_trg[me.m] && s.mask[i];
        if (!(s.surf[i] >= RSQR && considerme)) { ++n_disc; continue; }
        ++n_centre;
        nb.clear();
        gather(slabs, thr, i, R, RSQR, nb);
        n_pairs += nb.size();
        // counting sort of the ball by neighbour type (:3975-3997)
        std::fill(cs.begin(), cs.end(), 0);
        for (const Nb& q : nb) cs[q.m + 1]++;
        for (uint32_t ty = 0; ty < ntypes; ++ty) cs[ty + 1] += cs[ty];
        std::fill(fill.begin(), fill.end(), 0);
        ordered.resize(nb.size());
        for (const Nb& q : nb) ordered[cs[q.m] + fill[q.m]++] = q.d;
        for (int t = 0; t < ntasks; ++t) {
          if (!bit(trg_mask + 8 * t, me.m)) continue;
          const auto& env = env_types[t];
          if (doR) for (uint32_t ty : env) for (size_t k = cs[ty]; k < cs[ty + 1]; ++k) mR[t].add(ordered[k]);
          if (do1) {
            float closest = std::numeric_limits<float>::max();
            bool found = false;
            for (uint32_t ty : env) for (size_t k = cs[ty]; k < cs[ty + 1]; ++k)
              if (!(ordered[k] > closest)) { closest = ordered[k]; found = true; }
            m1[t].add(found ? closest : missing);
          }
          if (doK) for (uint32_t ty : env) for (size_t k = cs[ty]; k < cs[ty + 1]; ++k) mK[t].add(ordered[k]);
          if (doC) for (uint32_t ty : env) {
            const uint64_t c = cs[ty + 1] - cs[ty];
            if (c < cntnb_len) mC[t][c] += 1; else err = -3;
          }
          if (doM) {
            tmp.clear();
            for (uint32_t ty : env) for (size_t k = cs[ty]; k < cs[ty + 1]; ++k) tmp.push_back(ordered[k]);
            for (int kk = 0; kk < nk; ++kk) {
              const size_t ord = (size_t)k_list[kk] - 1;
              if (tmp.size() > ord) {
                std::nth_element(tmp.begin(), tmp.begin() + ord, tmp.end());
                mM[(size_t)t * nk + kk].add(tmp[ord]);
              } else {
                mM[(size_t)t * nk + kk].add(missing);
              }
            }
          }
        }
      }
#pragma omp barrier
    }
#pragma omp critical
    {
      for (int t = 0; t < ntasks; ++t) {
        if (doR) gR[t].merge(mR[t]);
        if (do1) g1[t].merge(m1[t]);
        if (doK) gK[t].merge(mK[t]);
        if (doC) for (uint64_t c = 0; c < cntnb_len; ++c) gC[t][c] += mC[t][c];
      }
      if (doM) for (size_t h = 0; h < gM.size(); ++h) gM[h].merge(mM[h]);
    }
  }
  const double t_comp1 = omp_get_wtime();
  if (err) return err;
  uint64_t o = 0;
  auto put = [&](const Hist& h) { for (uint64_t b = 0; b < H; ++b) out_bins[o++] = (uint64_t)h.cnt[b]; };
  if (doR) for (auto& h : gR) put(h);
  if (do1) for (auto& h : g1) put(h);
  if (doK) for (auto& h : gK) put(h);
  if (doM) for (auto& h : gM) put(h);
  if (doC) for (int t = 0; t < ntasks; ++t) std::memcpy(out_cntnb + (uint64_t)t * cntnb_len, gC[t].data(), cntnb_len * 8);
  if (stats) {
    stats[0] = n_centre; stats[1] = n_disc; stats[2] = n_pairs;
    stats[3] = (uint64_t)((t_build1 - t_build0) * 1e9);
    stats[4] = (uint64_t)((t_comp1 - t_build1) * 1e9);
  }
  return 0;
}

// Neighbour set of one ion: every j != centre with float d^2 <= R^2, sorted by
// (d^2, j) -- the tie order used to compare neighbour sets.
int ppo_neighbors(const float* xyz, uint64_t n, uint64_t centre, float R,
                  uint64_t* ids, float* d2, uint64_t cap, uint64_t* count) {
  if (!xyz || centre >= n || !count) return -1;
  const float r2 = R * R;
  const Ion me{xyz[3 * centre], xyz[3 * centre + 1], xyz[3 * centre + 2], 0};
  std::vector<std::pair<float, uint64_t>> v;
  for (uint64_t j = 0; j < n; ++j) {
    if (j == centre) continue;
    const Ion q{xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], 0};
    const float d = dist2(me, q);
    if (d <= r2) v.push_back({d, j});
  }
  std::sort(v.begin(), v.end());
  *count = v.size();
  for (uint64_t k = 0; k < v.size() && k < cap; ++k) { ids[k] = v[k].second; d2[k] = v[k].first; }
  return 0;
}

// The float category of one distance under histogram::add, exported so tests
// can check the device's bin-edge table against the CPU rounding.
// Occupancy grid of the whole cloud (vxlizer::rectangular_binning and the
// steps it calls, src/PARAPROBE_SolverHdl.cpp:5059-5386, :1471-1508, :1778-1791).
// bins[0..5] = vacuum, surface, inside voxels, nx, ny, nz.  Returns -1 when the
// grid has 2^32 voxels or more (the reference stops there too).
int ppo_voxelize(const float* xyz, uint64_t n, float w_min, float w_max, uint64_t* nions_inside,
                 float* volume_inside, uint64_t* bins) {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (uint64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      const float v = xyz[3 * i + k];
      if (v <= lo[k]) lo[k] = v;
      if (v >= hi[k]) hi[k] = v;
    }
  const float w = (float)(0.5 * (double)(w_min + w_max));
  uint64_t nv[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] -= w;
    hi[k] += w;
    nv[k] = (uint64_t)std::ceil((hi[k] - lo[k]) / w) + 2;
  }
  const uint64_t nx = nv[0], ny = nv[1], nz = nv[2], nxy = nx * ny, nxyz = nxy * nz;
  if (nx >= 0xffffffffull || ny >= 0xffffffffull || nz >= 0xffffffffull || nxyz >= 0xffffffffull) return -1;
  std::vector<uint32_t> occ(nxyz, 0);
  std::vector<uint64_t> bin(n);
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t c[3];
    for (int k = 0; k < 3; ++k) {
      const float t = (xyz[3 * i + k] - lo[k]) / w;
      const uint64_t sz = (uint64_t)t;
      c[k] = (sz != nv[k] - 1) ? 1 + sz : nv[k] - 1;
    }
    bin[i] = c[0] + c[1] * nx + c[2] * nxy;
    occ[bin[i]] += 1;
  }
  // outer vacuum: the cluster of the corner (0, 0, nz - 1) among the empty
  // voxels, labelled in raster order with the reference's rules
  // (src/PARAPROBE_HoshenKopelman.cpp:55-146): a voxel joins the clusters of
  // its labelled -x, -y, -z neighbours, except that with all three labelled
  // only -y and -z are merged; voxel 0 carries label 0 and so stays unlabelled
  std::vector<uint32_t> uf(nxyz);
  for (uint64_t b = 0; b < nxyz; ++b) uf[b] = (uint32_t)b;
  auto root = [&](uint32_t a) {
    while (uf[a] != a) { uf[a] = uf[uf[a]]; a = uf[a]; }
    return a;
  };
  auto unite = [&](uint32_t a, uint32_t b) {
    a = root(a); b = root(b);
    if (a != b) uf[a] = b;
  };
  auto labelled = [&](uint64_t b) { return b != 0 && occ[b] == 0; };
  for (uint64_t z = 0; z < nz; ++z)
    for (uint64_t y = 0; y < ny; ++y)
      for (uint64_t x = 0; x < nx; ++x) {
        const uint64_t v = x + y * nx + z * nxy;
        if (!labelled(v)) continue;
        const bool L = x > 0 && labelled(v - 1), B = y > 0 && labelled(v - nx), F = z > 0 && labelled(v - nxy);
        if (L && B && F) { unite(v - nx, v - nxy); unite(v, v - nx); continue; }
        if (L) unite(v, v - 1);
        if (B) unite(v, v - nx);
        if (F) unite(v, v - nxy);
      }
  std::vector<char> vac(nxyz, 0);
  const uint64_t corner = (nz - 1) * nxy;
  if (labelled(corner)) {
    const uint32_t rc = root((uint32_t)corner);
    for (uint64_t b = 0; b < nxyz; ++b) vac[b] = labelled(b) && root((uint32_t)b) == rc;
  }
  // surface: non-vacuum Moore neighbours of vacuum voxels off the grid border
  std::vector<char> srf(nxyz, 0);
  for (uint64_t z = 1; z + 1 < nz; ++z)
    for (uint64_t y = 1; y + 1 < ny; ++y)
      for (uint64_t x = 1; x + 1 < nx; ++x) {
        if (!vac[x + y * nx + z * nxy]) continue;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const uint64_t t = (x + dx) + (y + dy) * nx + (z + dz) * nxy;
              if ((dx || dy || dz) && !vac[t]) srf[t] = 1;
            }
      }
  uint64_t nv_b = 0, ns_b = 0, ni_b = 0, nin = 0;
  for (uint64_t b = 0; b < nxyz; ++b) {
    nv_b += vac[b];
    ns_b += srf[b];
    if (!vac[b] && !srf[b]) { ++ni_b; nin += occ[b]; }
  }
  float vol = (float)ni_b;
  vol *= w * w * w;
  if (nions_inside) *nions_inside = nin;
  if (volume_inside) *volume_inside = vol;
  if (bins) { bins[0] = nv_b; bins[1] = ns_b; bins[2] = ni_b; bins[3] = nx; bins[4] = ny; bins[5] = nz; }
  return 0;
}

// n-point correlations (AnalysisSpatDistrType 5): for every centre (the
// filter of ppo_spatstat) and every task whose targets hold its type, the
// (order+1)-th nearest environment neighbour within R -- by (d^2, ion index)
// -- contributes its difference vector (neighbour minus centre) to the task's
// cubic histogram, binned as npc3d::add does (src/PARAPROBE_SolverHdl.cpp:
// 3899-3955, src/PARAPROBE_NPointCorrelations3D.cpp:48-160).  out holds
// ntasks * edge^3 uint32 counts; *edge_out = edge.  Returns -2 if out_cap is
// too small.  (The reference takes the element nth_element places at order,
// so among exact distance ties its pick is arbitrary; here ties go to the
// lower ion index.)
int ppo_npcorr(const float* xyz, const uint8_t* label, const float* ion2surf, uint64_t n, float rincr, float rmax,
               int ntasks, const uint32_t* trg_mask, const uint32_t* env_mask, uint32_t order, uint32_t* out,
               uint64_t out_cap, uint64_t* edge_out) {
  const uint64_t half = (uint64_t)(std::ceil(rmax / rincr) + 1.f);
  const uint64_t edge = 1 + 2 * half, nxy = edge * edge, nxyz = nxy * edge;
  if (edge_out) *edge_out = edge;
  if ((uint64_t)ntasks * nxyz > out_cap) return -2;
  std::fill(out, out + (uint64_t)ntasks * nxyz, 0u);
  const float R = rmax, RSQR = R * R, inv = 1.f / rincr;
  std::vector<uint8_t> any_trg(256, 0);
  for (int t = 0; t < ntasks; ++t)
    for (uint32_t ty = 0; ty < 256; ++ty) if (bit(trg_mask + 8 * t, ty)) any_trg[ty] = 1;
  // neighbour search on a uniform grid of edge R
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (uint64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], xyz[3 * i + k]); hi[k] = std::max(hi[k], xyz[3 * i + k]); }
  int64_t g[3];
  for (int k = 0; k < 3; ++k) g[k] = std::max<int64_t>(1, (int64_t)((hi[k] - lo[k]) / R) + 1);
  auto cell_of = [&](uint64_t i, int k) {
    return std::min<int64_t>(g[k] - 1, std::max<int64_t>(0, (int64_t)((xyz[3 * i + k] - lo[k]) / R)));
  };
  std::vector<std::vector<uint64_t>> cells((size_t)(g[0] * g[1] * g[2]));
  for (uint64_t i = 0; i < n; ++i)
    cells[(size_t)((cell_of(i, 2) * g[1] + cell_of(i, 1)) * g[0] + cell_of(i, 0))].push_back(i);
  struct Cand { float d2; uint64_t j; };
#pragma omp parallel
  {
    std::vector<Cand> nb, tmp;
    std::vector<uint32_t> mine((uint64_t)ntasks * nxyz, 0u);
#pragma omp for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
      const uint64_t i = (uint64_t)ii;
      if (!any_trg[label[i]] || !(ion2surf[i] >= RSQR)) continue;
      nb.clear();
      const int64_t c0 = cell_of(i, 0), c1 = cell_of(i, 1), c2 = cell_of(i, 2);
      for (int64_t z = std::max<int64_t>(0, c2 - 1); z <= std::min<int64_t>(g[2] - 1, c2 + 1); ++z)
        for (int64_t y = std::max<int64_t>(0, c1 - 1); y <= std::min<int64_t>(g[1] - 1, c1 + 1); ++y)
          for (int64_t x = std::max<int64_t>(0, c0 - 1); x <= std::min<int64_t>(g[0] - 1, c0 + 1); ++x)
            for (uint64_t j : cells[(size_t)((z * g[1] + y) * g[0] + x)]) {
              if (j == i) continue;
              const float dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1],
                          dz = xyz[3 * i + 2] - xyz[3 * j + 2];
              const float d2 = (dx * dx + dy * dy) + dz * dz;
              if (d2 <= RSQR) nb.push_back({d2, j});
            }
      for (int t = 0; t < ntasks; ++t) {
        if (!bit(trg_mask + 8 * t, label[i])) continue;
        tmp.clear();
        for (const Cand& c : nb) if (bit(env_mask + 8 * t, label[c.j])) tmp.push_back(c);
        if (tmp.size() <= order) continue;
        std::nth_element(tmp.begin(), tmp.begin() + order, tmp.end(), [](const Cand& a, const Cand& b) {
          return a.d2 < b.d2 || (a.d2 == b.d2 && a.j < b.j);
        });
        const uint64_t j = tmp[order].j;
        const float u = xyz[3 * j] - xyz[3 * i], v = xyz[3 * j + 1] - xyz[3 * i + 1], w = xyz[3 * j + 2] - xyz[3 * i + 2];
        const float d = std::sqrt((u * u + v * v) + w * w);
        if (!(d <= R)) continue;
        int64_t b[3];
        const float comp[3] = {u, v, w};
        for (int k = 0; k < 3; ++k) {
          const float there = comp[k] * inv;
          const int disc = (there >= 0.f) ? (int)((double)there + 0.5) : (int)((double)there - 0.5);
          b[k] = disc + (int64_t)half;
        }
        mine[(uint64_t)t * nxyz + (uint64_t)(b[0] + b[1] * (int64_t)edge + b[2] * (int64_t)nxy)] += 1;
      }
    }
#pragma omp critical
    for (uint64_t k = 0; k < mine.size(); ++k) out[k] += mine[k];
  }
  return 0;
}

// Statistics after clustering (src/PARAPROBE_SolverHdl.cpp:4790-4945).
// clustered[i] != 0 marks a cluster member.  Guard zone: every unclustered ion
// within R (float d^2 <= R^2) of a clustered ion -- the intended rule; the
// reference's loop flags ions_kdtree.at(cand), the candidate's position in
// its result list, instead of the candidate (:4807-4815).  Centres:
// unclustered, unguarded ions with ion2surf >= R^2; neighbours: unclustered
// ions of any type.  RDF and RIPK add every neighbour distance, 1NN the
// smallest one and nothing without one (:4886-4913).  out: [RDF][1NN][RIPK]
// histograms (each present when asked), H = nbins + 2 uint64 each;
// stats = {centres, guard ions, centres without a neighbour}.
//
// guard_mode 1 restates the guard loop as the reference runs it
// (:4804-4820): positions are the input order (the reference's ions_kdtree
// order); for every position i, in order, whose ion is clustered -- flagged,
// or relabelled by an earlier step -- the loop reads ions_kdtree.at(cand) for
// cand = 0 .. |ball(i)| - 1 and gives every unclustered one i's clustered type
// (flag_as_guarded leaves a clustered type as it is, :4576-4582).  Those ions
// are clustered from then on: excluded as centres and as neighbours; the guard
// count is the number of relabellings.
int ppo_aposteriori(const float* xyz, const uint8_t* clustered, const float* ion2surf, uint64_t n, float rmin,
                    float rincr, float rmax, uint32_t analyses, int guard_mode, uint64_t* out, uint64_t out_cap,
                    uint64_t* stats) {
  if (!xyz || !clustered || !ion2surf || !out) return -1;
  Hist proto; proto.init(rmin, rincr, rmax);
  const uint64_t H = proto.nbins + 2;
  const bool doR = analyses & A_RDF, do1 = analyses & A_1NN, doK = analyses & A_RIPK;
  if (H * ((doR ? 1 : 0) + (do1 ? 1 : 0) + (doK ? 1 : 0)) > out_cap) return -2;
  const float R = rmax, RSQR = R * R;
  // uniform grid with cells a little wider than R: the +-1 cell stencil holds
  // every neighbour within R whatever the rounding of the cell coordinates
  const float h = R * 1.001f;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (uint64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], xyz[3 * i + k]); hi[k] = std::max(hi[k], xyz[3 * i + k]); }
  int64_t g[3];
  for (int k = 0; k < 3; ++k) g[k] = n ? std::max<int64_t>(1, (int64_t)((hi[k] - lo[k]) / h) + 1) : 1;
  auto cell_of = [&](uint64_t i, int k) {
    return std::min<int64_t>(g[k] - 1, std::max<int64_t>(0, (int64_t)((xyz[3 * i + k] - lo[k]) / h)));
  };
  std::vector<std::vector<uint64_t>> cells((size_t)(g[0] * g[1] * g[2]));
  for (uint64_t i = 0; i < n; ++i)
    cells[(size_t)((cell_of(i, 2) * g[1] + cell_of(i, 1)) * g[0] + cell_of(i, 0))].push_back(i);
  auto each_nb = [&](uint64_t i, auto&& f) {
    const int64_t c0 = cell_of(i, 0), c1 = cell_of(i, 1), c2 = cell_of(i, 2);
    for (int64_t z = std::max<int64_t>(0, c2 - 1); z <= std::min<int64_t>(g[2] - 1, c2 + 1); ++z)
      for (int64_t y = std::max<int64_t>(0, c1 - 1); y <= std::min<int64_t>(g[1] - 1, c1 + 1); ++y)
        for (int64_t x = std::max<int64_t>(0, c0 - 1); x <= std::min<int64_t>(g[0] - 1, c0 + 1); ++x)
          for (uint64_t j : cells[(size_t)((z * g[1] + y) * g[0] + x)]) {
            if (j == i) continue;
            const float dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1],
                        dz = xyz[3 * i + 2] - xyz[3 * j + 2];
            const float d2 = (dx * dx + dy * dy) + dz * dz;
            if (d2 <= RSQR) f(j, d2);
          }
  };
  std::vector<uint8_t> guard(n, 0);
  std::vector<uint8_t> excl(clustered, clustered + n);  // clustered types
  uint64_t ncent = 0, nlost = 0, nguard = 0;
  if (guard_mode == 1) {
    for (uint64_t i = 0; i < n; ++i) {
      if (!excl[i]) continue;
      uint64_t candidates = 0;
      each_nb(i, [&](uint64_t, float) { ++candidates; });
      for (uint64_t cand = 0; cand < candidates; ++cand) {
        if (excl[cand]) continue;
        excl[cand] = 1;
        ++nguard;
      }
    }
  } else {
    for (uint64_t i = 0; i < n; ++i)
      if (clustered[i]) each_nb(i, [&](uint64_t j, float) { if (!clustered[j]) guard[j] = 1; });
    for (uint64_t i = 0; i < n; ++i) nguard += guard[i];
  }
  const uint8_t* clus = excl.data();
  Hist hR = proto, h1 = proto, hK = proto;
#pragma omp parallel
  {
    Hist mR = proto, m1 = proto, mK = proto;
    uint64_t myc = 0, myl = 0;
#pragma omp for schedule(dynamic, 256)
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
      const uint64_t i = (uint64_t)ii;
      if (!(ion2surf[i] >= RSQR) || clus[i] || guard[i]) continue;
      ++myc;
      float closest = FLT_MAX;
      bool any = false;
      each_nb(i, [&](uint64_t j, float d2) {
        if (clus[j]) return;
        const float d = std::sqrt(d2);
        if (doR) mR.add(d);
        if (doK) mK.add(d);
        if (d <= closest) { closest = d; any = true; }
      });
      if (do1) { if (any) m1.add(closest); else ++myl; }
    }
#pragma omp critical
    {
      hR.merge(mR); h1.merge(m1); hK.merge(mK);
      ncent += myc; nlost += myl;
    }
  }
  uint64_t o = 0;
  auto put = [&](const Hist& hh) { for (uint64_t b = 0; b < H; ++b) out[o++] = (uint64_t)hh.cnt[b]; };
  if (doR) put(hR);
  if (do1) put(h1);
  if (doK) put(hK);
  if (stats) { stats[0] = ncent; stats[1] = nguard; stats[2] = nlost; }
  return 0;
}

int ppo_category(float rmin, float rincr, float rmax, float x) {
  Hist h; h.init(rmin, rincr, rmax);
  double xx = x;
  if (xx >= h.start && xx <= h.end) {
    float rb = (float)((xx - h.start) * h.scale);
    uint32_t b = (uint32_t)std::floor(rb);
    return b < h.nbins ? (int)(1 + b) : (int)(h.nbins + 1);
  }
  if (xx < h.start) return 0;
  if (xx > h.end) return (int)(h.nbins + 1);
  return -1;
}

}  // extern "C"
