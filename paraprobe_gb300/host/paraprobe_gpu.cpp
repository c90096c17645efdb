// paraprobe_gpu.cpp -- drop-in command line for PARAPROBE's descriptive
// spatial statistics on a GB300:
//
//   paraprobe_gpu <simid> <settings.xml> [--outdir DIR] [--device N]
//                 [--inside NIONS VOLUME] [--labels FILE] [--plan]
//                 [--fp64-audit CENTRES]
//
// Follows the reference's flow for this task (src/PARAPROBE_Main.cpp:100-305
// -> solver::characterize_spatstat, src/PARAPROBE_SolverHdl.cpp:745-776):
// read and check the settings, load the POS file, range it with the RRNG file
// (on the device), attach the VTK hull, parse the tasks, run the statistics
// through the C ABI, and write the same CSV files.  With
// SpatStatAdditionalLabelRandomization = 1 a second pass runs with shuffled
// labels and writes the ".Rndmized" files.  The NumberOfIonsInside /
// VolumeInside values printed in the RDF header come from the reference's
// occupancy grid (pp_cloud_inside, voxel edge from AdvIonPruneBinWidthMin/Max);
// --inside supplies them instead.  --labels replays a given label
// assignment (one byte per ion, file order, e.g. a stored null-model shuffle)
// and writes ".Rndmized" files.  --plan prints the parsed task plan as JSON
// and runs nothing.  Every pass also recomputes the distances of a sample of
// centres (--fp64-audit CENTRES, evenly spaced; 0 = all; default 20000) in
// double precision, prints the largest error of the float arithmetic and
// writes PARAPROBE.SimID.<id>.FP64Audit.<Original|Rndmized>.csv, which lists
// every pair whose float bin or float in-ball decision differs from the
// double one together with the bin edge (or the cut-off R) it sits on.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "paraprobe_gb300.h"
#include "pp_io.h"

namespace {

void reporting(const std::string& w) { std::cout << "VERBOSE::" << w << std::endl; }
void stopping(const std::string& w) { std::cerr << "ERROR::" << w << std::endl; }

std::string json_escape(const std::string& s) {
  std::string o;
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
  }
  return o;
}

int check(pp_ctx* ctx, int rc, const char* what) {
  if (rc != PP_OK) stopping(std::string(what) + ": " + pp_strerror(rc) + ": " + pp_last_error(ctx));
  return rc;
}

// FP64 audit of the current tasks and bins: summary on stdout, and a CSV of
// every disagreement with the edge that explains it.  Bin edges are
// rmin + b (rmax - rmin) / nbins in double, the reference's histogram grid.
int fp64_audit(pp_ctx* ctx, int cloud, uint32_t centres, const ppio::Settings& S, uint64_t nbins,
               const std::string& outdir, bool randomized) {
  double max_abs = 0, max_rel = 0;
  uint64_t pairs = 0, bin_dis = 0, set_dis = 0, listed = 0;
  const uint64_t cap = 1u << 16;
  std::vector<uint64_t> ids(2 * cap);
  std::vector<double> dd(2 * cap);
  if (check(ctx, pp_fp64_audit(ctx, cloud, centres, &max_abs, &max_rel, &pairs, &bin_dis, &set_dis, ids.data(),
                               dd.data(), cap, &listed), "pp_fp64_audit"))
    return 7;
  std::cout << "FP64 audit (" << (centres ? std::to_string(centres) : std::string("all")) << " centres): " << pairs
            << " pairs, max abs error " << max_abs << " nm, max rel error " << max_rel << ", " << bin_dis
            << " bin and " << set_dis << " in-ball disagreements" << std::endl;
  const std::string fn = outdir + "/PARAPROBE.SimID." + std::to_string(S.sim_id) + ".FP64Audit." +
                         (randomized ? "Rndmized" : "Original") + ".csv";
  FILE* f = std::fopen(fn.c_str(), "w");
  if (!f) { stopping("cannot write " + fn); return 7; }
  std::fprintf(f, "MaxAbsError;%.18g\nMaxRelError;%.18g\nPairs;%llu\nBinDisagreements;%llu\nInBallDisagreements;%llu\n",
               max_abs, max_rel, (unsigned long long)pairs, (unsigned long long)bin_dis, (unsigned long long)set_dis);
  std::fprintf(f, "CentreIonID;NeighbourIonID;DistanceFloat;DistanceDouble;Edge;EdgeValue;DistanceToEdge\n");
  const double lo = (double)S.rmin, hi = (double)S.rmax, w = nbins ? (hi - lo) / (double)nbins : 0.0;
  for (uint64_t i = 0; i < listed && i < cap; ++i) {
    const double d64 = dd[2 * i + 1];
    long b = w > 0 ? (long)std::floor((d64 - lo) / w + 0.5) : 0;
    if (b < 0) b = 0;
    if ((uint64_t)b > nbins) b = (long)nbins;
    const double edge = lo + (double)b * w;
    const bool cut = std::fabs(d64 - hi) <= std::fabs(d64 - edge);
    std::fprintf(f, "%llu;%llu;%.18g;%.18g;%s;%.18g;%.18g\n", (unsigned long long)ids[2 * i],
                 (unsigned long long)ids[2 * i + 1], dd[2 * i], d64, cut ? "cutoff R" : ("bin edge " + std::to_string(b)).c_str(),
                 cut ? hi : edge, cut ? d64 - hi : d64 - edge);
  }
  std::fclose(f);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cerr << "usage: paraprobe_gpu <simid> <settings.xml> [--outdir DIR] [--device N] "
                 "[--inside NIONS VOLUME] [--labels FILE] [--plan] [--fp64-audit CENTRES]\n";
    return 2;
  }
  std::string outdir = ".";
  int device = 0;
  uint64_t nions_inside = 0;
  double volume_inside = 0.0;
  bool inside_given = false;
  bool plan_only = false;
  std::string labels_file;
  uint32_t audit_centres = 20000;
  for (int a = 3; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--outdir" && a + 1 < argc) outdir = argv[++a];
    else if (s == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else if (s == "--inside" && a + 2 < argc) {
      nions_inside = std::strtoull(argv[a + 1], nullptr, 10);
      volume_inside = std::strtod(argv[a + 2], nullptr);
      inside_given = true;
      a += 2;
    }
    else if (s == "--plan") plan_only = true;
    else if (s == "--labels" && a + 1 < argc) labels_file = argv[++a];
    else if (s == "--fp64-audit" && a + 1 < argc) audit_centres = (uint32_t)std::strtoul(argv[++a], nullptr, 10);
    else { std::cerr << "unknown option " << s << "\n"; return 2; }
  }
  ppio::Settings S;
  try {
    S = ppio::read_settings(argv[2]);
    S.sim_id = (unsigned int)std::stoul(argv[1]);
  } catch (std::exception& e) {
    stopping(std::string("Unable to parse control file! ") + e.what());
    return 3;
  }
  const std::string bad = ppio::check_settings(S);
  if (!bad.empty()) { stopping("Control file settings failed the validity check! " + bad); return 3; }
  if (!S.spatstat) { reporting("No spatial statistics task to do"); return 0; }
  if (S.input_format != 1 && !(S.input_format == 2 && S.recon_algo == 3)) {
    stopping("only POS input (InputFileformat 1) or EPOS input with its own coordinates (InputFileformat 2, "
             "ReconstructionAlgorithm 3) feeds this path");
    return 4;
  }
  if (S.surface_mode != 0 && S.surface_mode != 4) {
    stopping("only SurfaceReconstructionType 0 (none) or 4 (existing VTK hull) are provided");
    return 4;
  }

  ppio::Ranging rng;
  if (S.identify_ion_type && !ppio::read_rrng(S.rrng_file, rng)) std::cout << "WARNING::Unable to load RRNG file " << S.rrng_file << std::endl;
  const std::vector<ppio::Task> tasks = ppio::parse_tasks(S.tasks_code, rng);
  std::vector<uint32_t> ks;
  try {
    if (S.do_mknn) ks = ppio::mknn_orders(S.mknn_code);
  } catch (std::exception& e) {
    stopping(e.what());
    return 3;
  }
  uint32_t flags = (S.do_rdf ? PP_RDF : 0u) | (S.do_1nn ? PP_1NN : 0u) | (S.do_ripk ? PP_RIPK : 0u) |
                   (S.do_mknn ? PP_MKNN : 0u) | (S.do_cntnb ? PP_CNTNB : 0u) | (S.do_npcorr ? PP_NPCORR : 0u);
  if (S.do_npcorr) {
    // the reference skips the whole statistics task when the n-point
    // histogram would exceed 503^3 voxels (src/PARAPROBE_SolverHdl.cpp:3706-3712)
    const double edge = 1.0 + 2.0 * (double)(uint64_t)(std::ceil(S.rmax / S.rincr) + 1.f);
    if (edge * edge * edge > 503.0 * 503.0 * 503.0) {
      std::cout << "WARNING::Computation of 2-point statistics would require too large buffers, skipping!" << std::endl;
      return 0;
    }
  }
  if (plan_only) {
    std::cout << "{\"flags\": " << flags << ", \"rmin\": " << S.rmin << ", \"rincr\": " << S.rincr
              << ", \"rmax\": " << S.rmax << ", \"k\": [";
    for (size_t i = 0; i < ks.size(); ++i) std::cout << (i ? ", " : "") << ks[i];
    std::cout << "], \"max_type_id\": " << rng.max_type_id() << ", \"tasks\": [";
    for (size_t t = 0; t < tasks.size(); ++t) {
      std::cout << (t ? ", " : "") << "{\"trg\": [";
      size_t i = 0;
      for (auto& kv : tasks[t].trg) std::cout << (i++ ? ", " : "") << kv.second;
      std::cout << "], \"env\": [";
      i = 0;
      for (auto& kv : tasks[t].env) std::cout << (i++ ? ", " : "") << kv.second;
      std::cout << "], \"names\": [\"" << json_escape(tasks[t].trg_name()) << "\", \"" << json_escape(tasks[t].env_name())
                << "\"]}";
    }
    std::cout << "]}" << std::endl;
    return 0;
  }

  // ---- inputs
  std::vector<float> xyz, mq;
  // raw image for device ingest: big-endian (x, y, z, m/q) records, as a POS
  // file holds them (EPOS records are cut to their first 16 bytes)
  std::vector<uint8_t> raw;
  if (S.input_format == 2) {
    if (!ppio::read_epos_as_pos(S.raw_file, raw)) { stopping("File " + S.raw_file + " cannot be read!"); return 5; }
  } else {
    if (!ppio::read_pos(S.raw_file, xyz, mq)) { stopping("File " + S.raw_file + " cannot be read!"); return 5; }
    FILE* f = std::fopen(S.raw_file.c_str(), "rb");
    raw.resize(mq.size() * 16);
    const size_t got = f ? std::fread(raw.data(), 1, raw.size(), f) : 0;
    if (f) std::fclose(f);
    if (got != raw.size()) { stopping("I/O failed on " + S.raw_file); return 5; }
  }
  const uint64_t n = raw.size() / 16;
  std::vector<float> rlo, rhi;
  std::vector<uint8_t> rty;
  rng.flat(rlo, rhi, rty);
  std::vector<float> tri;
  const bool use_hull = S.surface_mode == 4 && S.debug_compute_distance;
  if (S.surface_mode == 4 && !ppio::read_vtk_hull(S.surface_file, tri)) {
    stopping("Unable to read the triangle hull " + S.surface_file);
    return 5;
  }

  pp_ctx* ctx = nullptr;
  if (pp_create(&ctx, device) != PP_OK) { stopping("no CUDA device"); return 6; }
  int cloud = -1;
  if (check(ctx, pp_cloud_upload_pos(ctx, raw.data(), n, rlo.data(), rhi.data(), rty.data(), (int)rty.size(), &cloud),
            "pp_cloud_upload_pos")) return 7;
  if (use_hull && check(ctx, pp_hull_upload(ctx, cloud, tri.data(), tri.size() / 9, S.carving_radius), "pp_hull_upload"))
    return 7;
  if (!use_hull) {
    // no hull or DebugComputeDistance = 0: every ion keeps R'^2
    const float rp = std::max(S.rmax, S.carving_radius);
    std::vector<float> d2(n, rp * rp);
    if (check(ctx, pp_surfdist_upload(ctx, cloud, d2.data()), "pp_surfdist_upload")) return 7;
  }
  if (!inside_given && S.do_rdf) {
    // the reference's TipBinning (vxlizer::rectangular_binning) supplies these
    float vol = 0.f;
    uint64_t vox[6] = {0, 0, 0, 0, 0, 0};
    if (check(ctx, pp_cloud_inside(ctx, cloud, S.bin_w_min, S.bin_w_max, &nions_inside, &vol, vox), "pp_cloud_inside"))
      return 7;
    volume_inside = vol;
    std::cout << "TipBinning with a nxyz grid " << vox[3] << ";" << vox[4] << ";" << vox[5] << ": " << vox[0]
              << " vacuum, " << vox[1] << " surface, " << vox[2] << " inside bins, " << nions_inside
              << " ions inside" << std::endl;
  }
  const int nt = (int)tasks.size();
  std::vector<uint32_t> trg(8 * (size_t)nt, 0), env(8 * (size_t)nt, 0);
  for (int t = 0; t < nt; ++t) {
    for (auto& kv : tasks[t].trg) trg[8 * t + (kv.second >> 5)] |= 1u << (kv.second & 31);
    for (auto& kv : tasks[t].env) env[8 * t + (kv.second >> 5)] |= 1u << (kv.second & 31);
  }
  if (check(ctx, pp_tasks_set(ctx, trg.data(), env.data(), nt), "pp_tasks_set")) return 7;
  if (check(ctx, pp_hist_params(ctx, S.rmin, S.rincr, S.rmax), "pp_hist_params")) return 7;
  if (S.do_npcorr && check(ctx, pp_set_option(ctx, "npcorr_order", (int)S.knn_order), "pp_set_option")) return 7;
  const uint32_t fl_run = flags & ~(uint32_t)((S.do_mknn && ks.empty()) ? PP_MKNN : 0u);

  auto pass = [&](const uint32_t* perm, bool randomized) -> int {
    if (check(ctx, pp_run(ctx, cloud, fl_run, ks.data(), (int)ks.size(), perm, nullptr), "pp_run")) return 7;
    uint64_t total = 0, nb = 0;
    if (check(ctx, pp_result_size(ctx, &total, &nb), "pp_result_size")) return 7;
    std::vector<uint64_t> bins(std::max<uint64_t>(total, 1));
    if (check(ctx, pp_fetch(ctx, bins.data(), bins.size()), "pp_fetch")) return 7;
    uint64_t centres = 0, discarded = 0, pairs = 0;
    pp_run_stats(ctx, &centres, &discarded, &pairs);
    std::cout << "Descriptive spatial statistics considered/discarded " << centres << ";" << discarded << " ions, "
              << pairs << " neighbour pairs" << std::endl;
    if (fp64_audit(ctx, cloud, audit_centres, S, nb, outdir, randomized)) return 7;
    const uint64_t H = nb + 2;
    uint64_t o = 0;
    auto hist = [&](uint64_t at) {
      ppio::Histogram h{(double)S.rmin, (double)S.rincr, (uint32_t)nb, {}};
      h.counts.assign(bins.begin() + at, bins.begin() + at + H);
      return h;
    };
    std::vector<uint64_t> off_rdf, off_1nn, off_ripk;
    if (fl_run & PP_RDF) for (int t = 0; t < nt; ++t, o += H) off_rdf.push_back(o);
    if (fl_run & PP_1NN) for (int t = 0; t < nt; ++t, o += H) off_1nn.push_back(o);
    if (fl_run & PP_RIPK) for (int t = 0; t < nt; ++t, o += H) off_ripk.push_back(o);
    for (int t = 0; t < nt; ++t) {
      const std::string a = tasks[t].trg_name(), b = tasks[t].env_name();
      if (fl_run & PP_RDF) ppio::write_report(outdir, S.sim_id, ppio::Report::RDF, "RDF", a, b, hist(off_rdf[t]), randomized, nions_inside, volume_inside);
      if (fl_run & PP_1NN) ppio::write_report(outdir, S.sim_id, ppio::Report::NN1, "1NN", a, b, hist(off_1nn[t]), randomized, nions_inside, volume_inside);
      if (fl_run & PP_RIPK) ppio::write_report(outdir, S.sim_id, ppio::Report::RIPK, "RIPK", a, b, hist(off_ripk[t]), randomized, nions_inside, volume_inside);
    }
    if (fl_run & PP_MKNN)
      for (int t = 0; t < nt; ++t)
        for (size_t k = 0; k < ks.size(); ++k, o += H)
          ppio::write_report(outdir, S.sim_id, ppio::Report::MKNN, "MKNN" + std::to_string(ks[k]), tasks[t].trg_name(),
                             tasks[t].env_name(), hist(o), randomized, nions_inside, volume_inside);
    if (fl_run & PP_NPCORR) {
      // the reference writes these histograms to HDF5; here one raw file of
      // edge^3 uint32 counts ([z][y][x], voxel size SpatStatRadiusIncr) per task
      uint64_t e = 0;
      if (check(ctx, pp_fetch_npcorr(ctx, nullptr, 0, &e), "pp_fetch_npcorr")) return 7;
      const uint64_t per = e * e * e;
      std::vector<uint32_t> cnt(std::max<uint64_t>(per * nt, 1));
      if (check(ctx, pp_fetch_npcorr(ctx, cnt.data(), cnt.size(), &e), "pp_fetch_npcorr")) return 7;
      for (int t = 0; t < nt; ++t) {
        const std::string fn = outdir + "/PARAPROBE.SimID." + std::to_string(S.sim_id) + ".NPCORR." +
                               tasks[t].trg_name() + "." + tasks[t].env_name() + "." +
                               (randomized ? "Rndmized" : "Original") + "." + std::to_string(e) + "x" +
                               std::to_string(e) + "x" + std::to_string(e) + ".u32";
        FILE* f = std::fopen(fn.c_str(), "wb");
        if (!f || std::fwrite(cnt.data() + (size_t)t * per, 4, per, f) != per) {
          if (f) std::fclose(f);
          stopping("cannot write " + fn);
          return 7;
        }
        std::fclose(f);
      }
    }
    if (fl_run & PP_CNTNB) {
      uint64_t L = 0;
      if (check(ctx, pp_fetch_cntnb(ctx, nullptr, 0, &L), "pp_fetch_cntnb")) return 7;
      std::vector<uint64_t> cn(std::max<uint64_t>(L * nt, 1));
      if (check(ctx, pp_fetch_cntnb(ctx, cn.data(), cn.size(), &L), "pp_fetch_cntnb")) return 7;
      for (int t = 0; t < nt; ++t) {
        std::vector<uint64_t> c(cn.begin() + (size_t)t * L, cn.begin() + (size_t)(t + 1) * L);
        while (!c.empty() && c.back() == 0) c.pop_back();
        ppio::write_nbcnt(outdir, S.sim_id, tasks[t].trg_name(), tasks[t].env_name(), c, randomized);
      }
    }
    return 0;
  };
  // a permutation that gives ion i the label target[i] (pp_run's label_perm):
  // every target label is matched to a distinct ion of that type, in order
  auto perm_for = [&](const std::vector<uint8_t>& current, const std::vector<uint8_t>& target,
                      std::vector<uint32_t>& perm) -> bool {
    std::vector<std::vector<uint32_t>> by_type(256);
    for (uint64_t i = 0; i < n; ++i) by_type[current[i]].push_back((uint32_t)i);
    std::vector<size_t> next(256, 0);
    perm.resize(n);
    for (uint64_t i = 0; i < n; ++i) {
      if (next[target[i]] >= by_type[target[i]].size()) return false;
      perm[i] = by_type[target[i]][next[target[i]]++];
    }
    return true;
  };
  if (!labels_file.empty()) {
    std::vector<uint8_t> lab(n), given(n);
    FILE* f = std::fopen(labels_file.c_str(), "rb");
    const size_t got = f ? std::fread(given.data(), 1, n, f) : 0;
    if (f) std::fclose(f);
    if (got != n) { stopping("cannot read " + labels_file); pp_destroy(ctx); return 5; }
    if (check(ctx, pp_cloud_labels(ctx, cloud, lab.data(), n), "pp_cloud_labels")) return 7;
    std::vector<uint32_t> perm;
    if (!perm_for(lab, given, perm)) { stopping("--labels does not permute the ranged labels"); pp_destroy(ctx); return 5; }
    const int rc = pass(perm.data(), true);
    pp_destroy(ctx);
    return rc;
  }
  int rc = pass(nullptr, false);
  if (rc == 0 && S.label_rnd) {
    // null model: permute the labels of all ions once (deterministic shuffle)
    std::vector<uint8_t> lab(n), shuffled(n);
    if (check(ctx, pp_cloud_labels(ctx, cloud, lab.data(), n), "pp_cloud_labels")) return 7;
    std::vector<uint32_t> idx;
    pp_shuffle_labels(lab.data(), n, S.rnd_seed, shuffled.data());
    perm_for(lab, shuffled, idx);
    rc = pass(idx.data(), true);
  }
  pp_destroy(ctx);
  return rc;
}
