// ref_harness.cpp -- drives the REFERENCE's own compiled units (test only).
//
// Built by oracle/ref/Makefile from the read-only reference tree into
// oracle/_ref/ref_spatstat.  It links PARAPROBE's unmodified KDTree.cpp,
// Math.cpp, AABBTree.cpp, PeriodicTable.cpp, Settings.cpp and Datatypes.cpp
// and uses its header-only histogram/discrhistogram/pos classes.  The glue
// that lives in src/PARAPROBE_SolverHdl.cpp (which cannot be compiled here:
// CGAL, HDF5, voro++, MKL) is restated in this file, following the cited
// lines, so that the arithmetic that decides every count -- ranging, task
// parsing, settings parsing, KD-tree ball queries, histogram::add, AABB tree
// queries and closestPointOnTriangle -- is the reference's own code.
//
// Usage:
//   ref_spatstat <simid> <settings.xml> <nthreads> <outdir>
//                [--labels <file of uint8 per ion, original order>]
//                [--inside <nions_inside> <volume_inside>]
//                [--voxelize]
//                [--dump-surf]
//                [--aposteriori <flags file: uint8 per ion, nonzero = clustered> <rdf|1nn|ripk>]
// Writes into <outdir>:
//   the reference CSV files (report_apriori_descrstat2/3 layout),
//   raw_bins.u64    uint64 counts, layout of pp_fetch (RDF,1NN,RIPK,MKNN groups)
//   raw_cntnb.u64   uint64 [ntasks][L] neighbour-count histogram, L in stats
//   stats.txt       centres, discarded, pairs, nbins, ntasks, nk, L
//   ion2surf.f32    (with --dump-surf) squared hull distance per original ion
//   raw_npcorr.u32  (AnalysisSpatDistrType 5) uint32 [ntasks][edge^3] n-point
//                   correlation counts of the reference's npc3d class
//   raw_apost.u64   (with --aposteriori, one thread) the histogram of the
//                   statistics after clustering, H = nbins + 2 counts
//   tree_order.u64  (with --aposteriori) the order of the clustering task's
//                   global KD-tree: position p holds original ion tree_order[p]
//   apost_stats.txt (with --aposteriori) guarded ions, centres, centres
//                   without a neighbour
//   voxel.txt       (with --voxelize) the occupancy grid's NumberOfIonsInside and
//                   VolumeInside, which then also head the RDF reports; the
//                   Hoshen-Kopelman clustering is the reference's percAnalyzer
// The process runs everything single-rank; nthreads selects the z-slab count
// (one KD-tree per slab) exactly as OMP_NUM_THREADS does in the reference.

#include "PARAPROBE_KDTree.h"
#include "PARAPROBE_DiscreteHistogram.h"
#include "PARAPROBE_HoshenKopelman.h"
#include "PARAPROBE_NPointCorrelations3D.h"

#include <omp.h>
#include <sys/stat.h>

#include <cstdint>
#include <cstdio>

using namespace std;

// The reference's logging helpers live in src/PARAPROBE_Main.cpp:75-96.
void reporting(const int rank, const string what) { cout << "VERBOSE::" << rank << " " << what << endl; }
void reporting(const string what) { cout << "VERBOSE::" << what << endl; }
void complaining(const int rank, const string what) { cout << "WARNING::" << rank << " " << what << endl; }
void complaining(const string what) { cout << "WARNING::" << what << endl; }
void stopping(const int rank, const string what) { cerr << "ERROR::" << rank << " " << what << endl; }
void stopping(const string what) { cerr << "ERROR::" << what << endl; }

namespace {

// Type flags of the statistics after clustering (src/PARAPROBE_HPDBScan.cpp:1105-1111,
// src/PARAPROBE_SolverHdl.cpp:4576-4621), free functions of files that do not
// compile here, restated.
unsigned int flag_as_clustered(const unsigned int typid, const unsigned int maxtypid) {
  return typid <= maxtypid ? typid + ION_IN_CLUSTER : typid;
}
unsigned int flag_as_guarded(const unsigned int typid, const unsigned int maxtypid) {
  return typid <= maxtypid ? typid + ION_AT_CLUSTER : typid;
}
bool is_clustered(const unsigned int typid, const unsigned int maxtypid) {
  if (typid <= maxtypid + ION_IN_CLUSTER) return typid > maxtypid;
  return false;
}
bool is_guardzone(const unsigned int typid, const unsigned int maxtypid) {
  return typid > maxtypid + ION_IN_CLUSTER;
}

struct Region {
  apt_real zmi, zmx;
  vector<p3dm1> ions;        // ionpp3
  vector<apt_xyz> surf;      // ion2surf
  vector<p3dm1> ions_kd;     // ionpp3_kdtree
  vector<apt_xyz> surf_kd;   // ion2surf_kdtree
  vector<size_t> gid;        // original ion index (harness bookkeeping)
  vector<size_t> gid_kd;
  kd_tree* tree = nullptr;
};

bool read_pos(const string& fn, vector<pos>& out) {
  // src/PARAPROBE_SolverHdl.cpp:6797-6930 (block reads of big-endian records)
  FILE* f = fopen(fn.c_str(), "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (sz % (long)sizeof(pos_be_2_stl_le)) { fclose(f); return false; }
  size_t n = sz / sizeof(pos_be_2_stl_le);
  vector<pos_be_2_stl_le> raw(n);
  if (fread(raw.data(), sizeof(pos_be_2_stl_le), n, f) != n) { fclose(f); return false; }
  fclose(f);
  out.reserve(n);
  for (size_t i = 0; i < n; ++i) out.push_back(pos(raw[i]));
  return true;
}

bool read_vtk(const string& fn, vector<tri3d>& hull) {
  // src/PARAPROBE_SolverHdl.cpp:2029-2118: four header lines, "POINTS n ...",
  // then three vertex lines per triangle parsed with stof on ' ' tokens.
  ifstream f(fn.c_str());
  if (!f.is_open()) return false;
  string line, tok;
  for (int i = 0; i < 4; ++i) getline(f, line);
  getline(f, line);
  if (line.empty()) return false;
  istringstream ls(line);
  getline(ls, tok, ' ');
  getline(ls, tok, ' ');
  size_t nv = stoul(tok);
  if (nv % 3) return false;
  size_t v = 0;
  while (v < nv && f.good()) {
    tri3d t;
    apt_real* c[9] = {&t.x1, &t.y1, &t.z1, &t.x2, &t.y2, &t.z2, &t.x3, &t.y3, &t.z3};
    for (int k = 0; k < 3; ++k) {
      getline(f, line);
      istringstream s(line);
      for (int q = 0; q < 3; ++q) { getline(s, tok, ' '); *c[3 * k + q] = stof(tok.c_str()); }
    }
    hull.push_back(t);
    v += 3;
  }
  return v == nv;
}

string task_names(const map<string, unsigned int>& m) {
  string s;
  for (auto& kv : m) s += kv.first;
  return s;
}

void report2(const string& outdir, long type, const string& what, const string& trg, const string& env,
             histogram& hist, bool rnd, size_t nions_inside, double volume_inside) {
  // src/PARAPROBE_SolverHdl.cpp:4299-4410
  string fn = outdir + "/PARAPROBE.SimID." + to_string(Settings::SimID) + "." + what + "." + trg + "." + env;
  fn += rnd ? ".Rndmized.csv" : ".Original.csv";
  ofstream sslog(fn.c_str());
  sslog.precision(18);
  double bend = hist.start() + hist.width();
  if (type == E_RDF) {
    sslog << "NumberOfIonsInside" << ";" << nions_inside << "\n";
    sslog << "VolumeInside" << ";" << volume_inside << " (nm^3)\n";
    if (volume_inside > EPSILON) {
      double globaldensity = static_cast<double>(nions_inside);
      globaldensity /= static_cast<double>(volume_inside);
      sslog << "InsideAtomicDensityEst" << ";" << globaldensity << "\n";
      double norm = (1.f / globaldensity) * (1.f / ((4.f / 3.f) * PI));
      sslog << "NormalizationFactor" << ";" << norm << "\n";
      sslog << "r;AccumulatedCount;nRDF(r);ShellVolume;RDF(r)\n";
      sslog << "nm;1;1;nm^3;1\n";
      sslog << "r;AccumulatedCount;nRDF(r);ShellVolume;RDF(r)\n";
      sslog << hist.start() << ";" << hist.cnts_lowest << ";;;\n";
      double half_dr = 0.5 * hist.width();
      for (unsigned int b = 0; b < hist.bincount(); ++b, bend += hist.width()) {
        double r = hist.start() + (0.5 + static_cast<double>(b)) * hist.width();
        double diff = (b > 0) ? (hist.report(b) - hist.report(b - 1)) : 0.f;
        double sphvol = CUBE(r + half_dr) - CUBE(r - half_dr);
        double rdfval = (sphvol > EPSILON) ? norm * diff / sphvol : 0.f;
        sslog << r << ";" << hist.report(b) << ";" << diff << ";" << sphvol << ";" << rdfval << "\n";
      }
      sslog << "" << ";" << hist.cnts_highest << ";;;\n";
    }
  }
  if (type == E_NEAREST_NEIGHBOR || type == E_MKNN) {
    if (type == E_NEAREST_NEIGHBOR) sslog << "1NN\n";
    if (type == E_MKNN) sslog << what << "\n";
    sslog << "BinEnd(r);Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
    sslog << "nm;1;1;1\n";
    sslog << "BinEnd(r);Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
    sslog << hist.start() << ";" << hist.cnts_lowest << ";;\n";
    double cum_sum = 0.f;
    for (unsigned int b = 0; b < hist.bincount(); ++b) cum_sum += hist.report(b);
    double sum = 0.f;
    for (unsigned int b = 0; b < hist.bincount(); ++b, bend += hist.width()) {
      sum += hist.report(b);
      double csum = (cum_sum > EPSILON) ? (sum / cum_sum) : 0.f;
      sslog << bend << ";" << hist.report(b) << ";" << sum << ";" << csum << "\n";
    }
    sslog << "" << ";" << hist.cnts_highest << ";;\n";
  }
  if (type == E_RIPLEYK) {
    sslog << "BinEnd(r);AccumulatedCounts\n";
    sslog << "nm;1\n";
    sslog << "BinEnd(r);AccumulatedCounts\n";
    sslog << hist.start() << ";" << hist.cnts_lowest << "\n";
    double sum = 0;
    for (unsigned int b = 0; b < hist.bincount(); ++b, bend += hist.width()) {
      sum += hist.report(b);
      sslog << bend << ";" << sum << "\n";
    }
    sslog << "" << ";" << hist.cnts_highest << "\n";
  }
}

void report3(const string& outdir, const string& trg, const string& env, discrhistogram& hist, bool rnd) {
  // src/PARAPROBE_SolverHdl.cpp:4412-4454
  string fn = outdir + "/PARAPROBE.SimID." + to_string(Settings::SimID) + ".NBCNTinRMAX." + trg + "." + env;
  fn += rnd ? ".Rndmized.csv" : ".Original.csv";
  ofstream sslog(fn.c_str());
  sslog.precision(18);
  sslog << "NeighborCountInRMax\n";
  sslog << "Value;Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
  sslog << "1;1;1;1\n";
  sslog << "Value;Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
  double cum_sum = 0.f;
  for (size_t b = 0; b < hist.cnts.size(); ++b) cum_sum += hist.cnts.at(b);
  double sum = 0.f;
  for (size_t b = 0; b < hist.cnts.size(); ++b) {
    sum += hist.cnts.at(b);
    double csum = (cum_sum > EPSILON) ? (sum / cum_sum) : 0.f;
    sslog << b << ";" << hist.cnts.at(b) << ";" << sum << ";" << csum << "\n";
  }
}

}  // namespace

// Occupancy grid of the whole cloud, restating vxlizer::rectangular_binning
// (src/PARAPROBE_SolverHdl.cpp:5342-5386) and the steps it calls: the tip box
// (:1778-1791), define_vxlgrid (:5318-5340), threadmemory::binning with
// rectangular_transfer (:1471-1508), binarization (:5272-5292),
// identify_vacuum_bins (:5196-5270, the reference's own percAnalyzer),
// identify_surface_adjacent_bins (:5132-5194), identify_inside_bins
// (:5115-5130) and characterize_binning (:5059-5112).
struct VoxelResult {
  size_t nions_inside = 0, vacuum = 0, surface = 0, inside = 0, nx = 0, ny = 0, nz = 0;
  apt_real volume_inside = 0.f;
};

static bool voxelize(const vector<pos>& raw, VoxelResult& out) {
  aabb3d tip = aabb3d();
  for (const pos& p : raw) {
    if (p.x <= tip.xmi) tip.xmi = p.x;
    if (p.x >= tip.xmx) tip.xmx = p.x;
    if (p.y <= tip.ymi) tip.ymi = p.y;
    if (p.y >= tip.ymx) tip.ymx = p.y;
    if (p.z <= tip.zmi) tip.zmi = p.z;
    if (p.z >= tip.zmx) tip.zmx = p.z;
  }
  tip.scale();
  const apt_xyz binwidth = 0.5 * (Settings::AdvIonPruneBinWidthMin + Settings::AdvIonPruneBinWidthMax);
  aabb3d ti = tip;
  const apt_real guardwidth = static_cast<apt_real>(binwidth);
  ti.blowup(guardwidth);
  const size_t nx = static_cast<size_t>(ceil((ti.xmx - ti.xmi) / binwidth)) + 2;
  const size_t ny = static_cast<size_t>(ceil((ti.ymx - ti.ymi) / binwidth)) + 2;
  const size_t nz = static_cast<size_t>(ceil((ti.zmx - ti.zmi) / binwidth)) + 2;
  const size_t nxy = nx * ny, nxyz = nxy * nz;
  if (nx >= UINT32MX || ny >= UINT32MX || nz >= UINT32MX || nxyz >= UINT32MX) return false;
  auto transfer = [](apt_xyz p, apt_xyz mi, apt_xyz w, size_t nvxl) {
    const apt_xyz tmpd = (p - mi) / w;
    const size_t tmpsz = static_cast<size_t>(tmpd);
    return (tmpsz != nvxl - 1) ? 1 + tmpsz : nvxl - 1;
  };
  vector<size_t> ion2bin(raw.size());
  for (size_t i = 0; i < raw.size(); ++i) {
    const size_t x = transfer(raw[i].x, ti.xmi, binwidth, nx);
    const size_t y = transfer(raw[i].y, ti.ymi, binwidth, ny);
    const size_t z = transfer(raw[i].z, ti.zmi, binwidth, nz);
    ion2bin[i] = x + y * nx + z * nxy;
  }
  vector<char> vac(nxyz, 0), srf(nxyz, 0), ins(nxyz, 0);
  bool* IsVacuum = new bool[nxyz];
  for (size_t b = 0; b < nxyz; ++b) IsVacuum[b] = false;
  for (size_t b : ion2bin) IsVacuum[b] = true;  // binarization: true = holds ions
  {
    percAnalyzer hk;
    if (!hk.initialize(IsVacuum, (unsigned int)nx, (unsigned int)ny, (unsigned int)nz) || !hk.hoshen_kopelman() ||
        !hk.compactify() || !hk.determine_clustersize_distr()) { delete[] IsVacuum; return false; }
    const unsigned int corner = 0 + 0 * (unsigned int)nx + ((unsigned int)nz - 1) * (unsigned int)nxy;
    if (!hk.rebinarize(corner, (unsigned int)nxyz, IsVacuum)) { delete[] IsVacuum; return false; }
  }
  for (size_t b = 0; b < nxyz; ++b) vac[b] = IsVacuum[b] ? 1 : 0;
  delete[] IsVacuum;
  for (size_t bz = 1; bz + 1 < nz; ++bz)
    for (size_t by = 1; by + 1 < ny; ++by)
      for (size_t bx = 1; bx + 1 < nx; ++bx) {
        if (!vac[bx + by * nx + bz * nxy]) continue;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              if (!dx && !dy && !dz) continue;
              const size_t there = (bx + dx) + (by + dy) * nx + (bz + dz) * nxy;
              if (!vac[there]) srf[there] = 1;
            }
      }
  for (size_t b = 0; b < nxyz; ++b) ins[b] = (!vac[b] && !srf[b]) ? 1 : 0;
  out = VoxelResult();
  for (size_t b : ion2bin) out.nions_inside += ins[b] ? 1 : 0;
  for (size_t b = 0; b < nxyz; ++b) { out.vacuum += vac[b]; out.surface += srf[b]; out.inside += ins[b]; }
  apt_real InsideVolume = static_cast<apt_real>(out.inside);
  InsideVolume *= CUBE(static_cast<apt_xyz>(binwidth));
  out.volume_inside = InsideVolume;
  out.nx = nx; out.ny = ny; out.nz = nz;
  return true;
}

int main(int argc, char** argv) {
  if (argc < 5) {
    cerr << "usage: ref_spatstat <simid> <settings.xml> <nthreads> <outdir> [--labels f] [--inside n v] [--dump-surf]\n";
    return 2;
  }
  Settings::SimID = stoul(argv[1]);
  Settings::readXML(argv[2]);
  if (!Settings::checkUserInput()) { cerr << "settings rejected\n"; return 3; }
  const int T = atoi(argv[3]);
  const string outdir = argv[4];
  string labels_fn;
  size_t nions_inside = 0;
  double volume_inside = 0.0;
  bool dump_surf = false, do_voxel = false;
  string apost_fn, apost_what;
  for (int a = 5; a < argc; ++a) {
    string s = argv[a];
    if (s == "--voxelize") { do_voxel = true; continue; }
    if (s == "--labels" && a + 1 < argc) labels_fn = argv[++a];
    else if (s == "--inside" && a + 2 < argc) { nions_inside = stoull(argv[a + 1]); volume_inside = stod(argv[a + 2]); a += 2; }
    else if (s == "--dump-surf") dump_surf = true;
    else if (s == "--aposteriori" && a + 2 < argc) { apost_fn = argv[a + 1]; apost_what = argv[a + 2]; a += 2; }
  }
  omp_set_num_threads(T);
  mkdir(outdir.c_str(), 0755);

  // ---- ingest + ranging (src/PARAPROBE_SolverHdl.cpp:6797-6930, :7340-7438)
  vector<pos> raw;
  if (!read_pos(Settings::RAWFilenameIn, raw)) { cerr << "cannot read POS\n"; return 4; }
  if (do_voxel) {
    VoxelResult v;
    if (!voxelize(raw, v)) { cerr << "voxelisation failed\n"; return 8; }
    nions_inside = v.nions_inside;
    volume_inside = v.volume_inside;
    ofstream vf((outdir + "/voxel.txt").c_str());
    vf.precision(18);
    vf << "nions_inside " << v.nions_inside << "\nvolume_inside " << v.volume_inside << "\nvacuum_bins " << v.vacuum
       << "\nsurface_bins " << v.surface << "\ninside_bins " << v.inside << "\nnx " << v.nx << "\nny " << v.ny
       << "\nnz " << v.nz << "\n";
  }
  PeriodicTable pse;
  if (!pse.read_rangefile2(Settings::RRNGFilenameIn)) { cerr << "cannot read RRNG\n"; return 5; }
  const size_t N = raw.size();
  vector<unsigned int> lbl(N);
  for (size_t i = 0; i < N; ++i) lbl[i] = pse.mq2ionname(raw[i].mq);
  bool rnd = false;
  if (!labels_fn.empty()) {
    FILE* f = fopen(labels_fn.c_str(), "rb");
    vector<uint8_t> l(N);
    if (!f || fread(l.data(), 1, N, f) != N) { cerr << "bad labels file\n"; return 6; }
    fclose(f);
    for (size_t i = 0; i < N; ++i) lbl[i] = l[i];
    rnd = true;
  }

  // ---- z-slab decomposition (src/PARAPROBE_SolverHdl.cpp:1819-1934)
  vector<apt_real> zc(N);
  for (size_t i = 0; i < N; ++i) zc[i] = raw[i].z;
  sort(zc.begin(), zc.end());
  vector<apt_real> qqss;
  for (int t = 1; t < T; ++t) qqss.push_back(static_cast<apt_real>(t) / static_cast<apt_real>(T));
  mathHdl mh;
  vector<apt_real> qq = mh.quantiles_nosort(zc, qqss);
  vector<Region> reg(T);
  for (int t = 0; t < T; ++t) {
    reg[t].zmi = (t == 0) ? (zc.at(0) - static_cast<apt_real>(AABBINCLUSION_EPSILON)) : qq.at(t - 1);
    reg[t].zmx = (t == T - 1) ? (zc.back() + static_cast<apt_real>(AABBINCLUSION_EPSILON)) : qq.at(t);
    for (size_t i = 0; i < N; ++i) {
      const p3dm1 p(raw[i].x, raw[i].y, raw[i].z, lbl[i]);
      if (p.z >= reg[t].zmi && p.z < reg[t].zmx) { reg[t].ions.push_back(p); reg[t].gid.push_back(i); }
    }
  }

  // ---- ion to hull distance (src/PARAPROBE_SolverHdl.cpp:312-479, :2690-2740)
  const apt_xyz Rp = max(Settings::SpatStatRadiusMax, Settings::SurfaceCellsCarvingRadius);
  const apt_xyz RpSQR = SQR(Rp);
  for (auto& r : reg) r.surf.assign(r.ions.size(), RpSQR);   // ion2surfdistance_init
  vector<tri3d> hull;
  if (Settings::SurfaceMeshingAlgo == E_LOADEXISTENTVTK) {
    if (!read_vtk(Settings::SurfaceFilenameIn, hull)) { cerr << "cannot read VTK\n"; return 7; }
  }
  if (!hull.empty() && Settings::DebugComputeDistance) {
    Tree* bvh = new Tree(static_cast<unsigned int>(hull.size()));
    unsigned int triid = 0;
    for (auto& t : hull) {
      apt_real xmi = fmin(fmin(t.x1, t.x2), t.x3), xmx = fmax(fmax(t.x1, t.x2), t.x3);
      apt_real ymi = fmin(fmin(t.y1, t.y2), t.y3), ymx = fmax(fmax(t.y1, t.y2), t.y3);
      apt_real zmi = fmin(fmin(t.z1, t.z2), t.z3), zmx = fmax(fmax(t.z1, t.z2), t.z3);
      bvh->insertParticle(triid++, trpl(xmi, ymi, zmi), trpl(xmx, ymx, zmx));
    }
    for (auto& r : reg) {
#pragma omp parallel for schedule(dynamic, 1)
      for (size_t i = 0; i < r.ions.size(); ++i) {
        mathHdl genius;
        p3d me(r.ions[i].x, r.ions[i].y, r.ions[i].z);
        AABB e_aabb(trpl(me.x - Rp, me.y - Rp, me.z - Rp), trpl(me.x + Rp, me.y + Rp, me.z + Rp));
        vector<unsigned int> cand = bvh->query(e_aabb);
        if (!cand.empty()) {
          apt_xyz best = RpSQR;
          for (unsigned int c : cand) {
            apt_xyz v = genius.closestPointOnTriangle(hull.at(c), me);
            if (v > best) continue;
            best = v;
          }
          r.surf[i] = best;
        }
      }
    }
    delete bvh;
  }
  if (dump_surf) {
    vector<float> s(N);
    for (auto& r : reg) for (size_t i = 0; i < r.ions.size(); ++i) s[r.gid[i]] = r.surf[i];
    FILE* f = fopen((outdir + "/ion2surf.f32").c_str(), "wb");
    fwrite(s.data(), 4, N, f);
    fclose(f);
  }

  if (!apost_fn.empty()) {
    if (T != 1) { cerr << "--aposteriori needs one thread (one region in input order)\n"; return 10; }
    // ---- statistics after clustering.  The cloud stands for the clustering
    // task's filtered ions (ions_filtered, :4665-4685) with the clustered ones
    // flagged by HPDBSCAN::summarize2 (flag_as_clustered).
    vector<uint8_t> cf(N);
    FILE* ff = fopen(apost_fn.c_str(), "rb");
    if (!ff || fread(cf.data(), 1, N, ff) != N) { cerr << "bad cluster flags file\n"; return 11; }
    fclose(ff);
    const unsigned int mxtypid = pse.get_maxtypeid();
    vector<p3dm1> ions_filtered = reg[0].ions;
    vector<apt_xyz> ion2surf_filtered = reg[0].surf;
    for (size_t i = 0; i < N; ++i)
      if (cf[i]) ions_filtered[i].m = flag_as_clustered(ions_filtered[i].m, mxtypid);
    // clustertask::build_kdtree (:4737-4787): the task's global KD-tree, the
    // ions repacked into its order
    vector<p3d> ioninput;
    for (auto& p : ions_filtered) ioninput.push_back(p3d(p.x, p.y, p.z));
    vector<size_t> permutations;
    kd_tree* globaltree = new kd_tree;
    globaltree->build(ioninput, permutations);
    vector<p3dm1> ions_kdtree;
    vector<apt_xyz> ion2surf_kdtree;
    globaltree->pack_p3dm1_d(permutations, ions_filtered, ion2surf_filtered, ions_kdtree, ion2surf_kdtree);
    if (!globaltree->verify(ions_kdtree)) { cerr << "KD-tree verify failed\n"; return 12; }
    // clustertask::flag2exclude_guard (:4790-4831), as written: the loop
    // reads and relabels ions_kdtree.at(cand), the candidate's position in
    // the result list, and gives it the clustered ion's (clustered) type
    apt_real Guard = Settings::SpatStatRadiusMax;
    apt_real SQRGuard = SQR(Guard);
    size_t guarded = 0;
    for (size_t i = 0; i < ions_kdtree.size(); ++i) {
      if (is_clustered(ions_kdtree.at(i).m, mxtypid) == true) {
        vector<size_t> candidates;
        globaltree->range_rball_noclear_nosort_indices(i, ions_kdtree, SQRGuard, candidates);
        for (size_t cand = 0; cand < candidates.size(); ++cand) {
          if (is_clustered(ions_kdtree.at(cand).m, mxtypid) == true) continue;
          ions_kdtree.at(cand).m = flag_as_guarded(ions_kdtree.at(i).m, mxtypid);
          ++guarded;
        }
      }
    }
    // clustertask::generic_spatstat (:4833-4945) for one analysis
    histogram globalres = histogram(Settings::SpatStatRadiusMin, Settings::SpatStatRadiusIncr, Settings::SpatStatRadiusMax);
    const apt_xyz R = Settings::SpatStatRadiusMax;
    const apt_xyz RSQR = SQR(R);
    size_t centres = 0, lost = 0;
    for (size_t i = 0; i < ions_kdtree.size(); ++i) {
      p3dm1 me = ions_kdtree.at(i);
      if (ion2surf_kdtree.at(i) >= RSQR && is_clustered(me.m, mxtypid) == false &&
          is_guardzone(me.m, mxtypid) == false) {
        vector<nbor> neighbors;
        globaltree->range_rball_noclear_nosort(i, ions_kdtree, RSQR, neighbors);
        ++centres;
        if (apost_what == "rdf" || apost_what == "ripk") {
          for (size_t nbb = 0; nbb < neighbors.size(); ++nbb)
            if (is_clustered(neighbors.at(nbb).m, mxtypid) == false) globalres.add(neighbors.at(nbb).d);
        } else if (apost_what == "1nn") {
          apt_real closest = F32MX;
          size_t nborid = numeric_limits<size_t>::max();
          for (size_t nbb = 0; nbb < neighbors.size(); ++nbb) {
            if (is_clustered(neighbors.at(nbb).m, mxtypid) == true) continue;
            if (neighbors.at(nbb).d > closest) continue;
            closest = neighbors.at(nbb).d;
            nborid = nbb;
          }
          if (nborid != numeric_limits<size_t>::max()) globalres.add(closest);
          else ++lost;
        }
      }
    }
    vector<uint64_t> hb;
    hb.push_back((uint64_t)globalres.cnts_lowest);
    for (size_t b = 0; b < globalres.bincount(); ++b) hb.push_back((uint64_t)globalres.cnts[b]);
    hb.push_back((uint64_t)globalres.cnts_highest);
    FILE* fo = fopen((outdir + "/raw_apost.u64").c_str(), "wb");
    fwrite(hb.data(), 8, hb.size(), fo);
    fclose(fo);
    vector<uint64_t> order(permutations.begin(), permutations.end());
    fo = fopen((outdir + "/tree_order.u64").c_str(), "wb");
    fwrite(order.data(), 8, order.size(), fo);
    fclose(fo);
    ofstream st((outdir + "/apost_stats.txt").c_str());
    st << "guarded " << guarded << "\ncentres " << centres << "\nlost " << lost << "\n";
    delete globaltree;
    return 0;
  }

  // ---- per-slab KD-trees (src/PARAPROBE_SolverHdl.cpp:1593-1663)
#pragma omp parallel for schedule(static, 1)
  for (int t = 0; t < T; ++t) {
    Region& r = reg[t];
    vector<p3d> in;
    for (auto& p : r.ions) in.push_back(p3d(p.x, p.y, p.z));
    vector<size_t> perm;
    r.tree = new kd_tree;
    r.tree->build(in, perm);
    r.tree->pack_p3dm1_dist(perm, r.ions, r.surf, r.ions_kd, r.surf_kd);
    for (size_t k = 0; k < perm.size(); ++k) r.gid_kd.push_back(r.gid[perm[k]]);
    if (!r.tree->verify(r.ions_kd)) cerr << "KD-tree verify failed\n";
  }

  // ---- tasks (src/PARAPROBE_SolverHdl.cpp:3019-3053)
  vector<TypeSpecDescrStat> tasks;
  parse_tasks(Settings::DescrStatTasksCode, tasks, pse);
  const size_t ntsk = tasks.size();

  // ---- compute_generic_spatstat3 (src/PARAPROBE_SolverHdl.cpp:3685-4177)
  vector<size_t> kcand;
  if (Settings::SpatStatDoMKNN && !Settings::DescrStatMKNNCode.empty() &&
      Settings::DescrStatMKNNCode.find('-') == string::npos) {
    istringstream line(Settings::DescrStatMKNNCode);
    string piece;
    int nsemi = count(Settings::DescrStatMKNNCode.begin(), Settings::DescrStatMKNNCode.end(), ';');
    for (int i = 0; i <= nsemi; ++i) {
      getline(line, piece, ';');
      if (!piece.empty() && piece.find_first_not_of("0123456789") == string::npos) {
        size_t val = stoul(piece);
        if (val < 1) { cerr << "k < 1\n"; return 8; }
        kcand.push_back(val - 1);
      }
    }
    sort(kcand.begin(), kcand.end(), [](size_t a, size_t b) { return a > b; });
  }
  const apt_real Rs = Settings::SpatStatRadiusMin, Ri = Settings::SpatStatRadiusIncr, Rm = Settings::SpatStatRadiusMax;
  vector<histogram> gR, g1, gK, gM;
  vector<discrhistogram> gC;
  for (size_t t = 0; t < ntsk; ++t) {
    if (Settings::SpatStatDoRDF) gR.push_back(histogram(Rs, Ri, Rm));
    if (Settings::SpatStatDo1NN) g1.push_back(histogram(Rs, Ri, Rm));
    if (Settings::SpatStatDoRIPK) gK.push_back(histogram(Rs, Ri, Rm));
    if (Settings::SpatStatDoCountNbors) gC.push_back(discrhistogram());
    if (Settings::SpatStatDoMKNN) for (size_t k = 0; k < kcand.size(); ++k) gM.push_back(histogram(Rs, Ri, Rm));
  }
  const unsigned int MaxTypes = pse.get_maxtypeid();
  // n-point correlations (src/PARAPROBE_SolverHdl.cpp:3706-3712, 3730-3736)
  const bool doP = Settings::SpatStatDoNPCorr;
  if (doP && npc3d(Rm, Ri, 0.f, false).get_support().nxyz > CUBE(MAXIMUM_NPC3D_BIN_RESOLUTION)) {
    cerr << "Computation of 2-point statistics would require too large buffers, skipping!\n";
    return 9;
  }
  vector<npc3d> gP;
  if (doP) for (size_t t = 0; t < ntsk; ++t) gP.push_back(npc3d(Rm, Ri, 0.f, true));
  const size_t KNNOrder = Settings::SpatStatKNNOrder;
  size_t centres = 0, discarded = 0, pairs = 0;
#pragma omp parallel reduction(+ : centres, discarded, pairs)
  {
    vector<histogram> mR, m1, mK, mM;
    vector<discrhistogram> mC;
    vector<npc3d> mP;
    if (doP) for (size_t t = 0; t < ntsk; ++t) mP.push_back(npc3d(Rm, Ri, 0.f, true));
    for (size_t t = 0; t < ntsk; ++t) {
      if (Settings::SpatStatDoRDF) mR.push_back(histogram(Rs, Ri, Rm));
      if (Settings::SpatStatDo1NN) m1.push_back(histogram(Rs, Ri, Rm));
      if (Settings::SpatStatDoRIPK) mK.push_back(histogram(Rs, Ri, Rm));
      if (Settings::SpatStatDoCountNbors) mC.push_back(discrhistogram());
      if (Settings::SpatStatDoMKNN) for (size_t k = 0; k < kcand.size(); ++k) mM.push_back(histogram(Rs, Ri, Rm));
    }
    for (int thr = 0; thr < T; ++thr) {
      vector<p3dm1> const& these = reg[thr].ions_kd;
      vector<apt_xyz>& dists = reg[thr].surf_kd;
      apt_xyz R = Settings::SpatStatRadiusMax;
      apt_xyz RSQR = SQR(R);
      kd_tree* kauri = reg[thr].tree;
#pragma omp for schedule(dynamic, 1) nowait
      for (size_t i = 0; i < these.size(); ++i) {
        p3dm1 me = these.at(i);
        bool considerme = false;
        for (auto& tk : tasks) {
          if (considerme) break;
          for (auto& kt : tk.trgcandidates) if (me.m == kt.second) { considerme = true; break; }
        }
        if (!(dists.at(i) >= RSQR && considerme)) { discarded++; continue; }
        centres++;
        vector<nbor> nb;
        kauri->range_rball_noclear_nosort(i, these, RSQR, nb);
        if (!((me.z - R) > reg[thr].zmi && (me.z + R) < reg[thr].zmx)) {
          for (int o = thr + 1; o < T; ++o) reg[o].tree->range_rball_noclear_nosort_external(me, reg[o].ions_kd, RSQR, nb);
          for (int o = thr - 1; o > -1; --o) reg[o].tree->range_rball_noclear_nosort_external(me, reg[o].ions_kd, RSQR, nb);
        }
        pairs += nb.size();
        if (doP) {
          // the KNNOrder-th environment neighbour's difference vector
          // (src/PARAPROBE_SolverHdl.cpp:3899-3955)
          vector<p3dm1> nb3;
          kauri->range_rball_noclear_nosort_p3dm1(i, these, RSQR, nb3);
          if (!((me.z - R) > reg[thr].zmi && (me.z + R) < reg[thr].zmx)) {
            for (int o = thr + 1; o < T; ++o)
              reg[o].tree->range_rball_noclear_nosort_external_p3dm1(me, reg[o].ions_kd, RSQR, nb3);
            for (int o = thr - 1; o > -1; --o)
              reg[o].tree->range_rball_noclear_nosort_external_p3dm1(me, reg[o].ions_kd, RSQR, nb3);
          }
          for (size_t t = 0; t < ntsk; ++t) {
            for (auto kt = tasks[t].trgcandidates.begin(); kt != tasks[t].trgcandidates.end(); ++kt) {
              if (me.m != kt->second) continue;
              if (nb3.size() > KNNOrder) {
                vector<npnbor> tmp;
                for (size_t nbb = 0; nbb < nb3.size(); ++nbb) {
                  for (auto jt = tasks[t].envcandidates.begin(); jt != tasks[t].envcandidates.end(); ++jt) {
                    if (nb3[nbb].m != jt->second) continue;
                    p3dm1 thisnb = nb3[nbb];
                    d3d diffv = d3d(thisnb.x - me.x, thisnb.y - me.y, thisnb.z - me.z);
                    apt_xyz dd = sqrt(SQR(diffv.u) + SQR(diffv.v) + SQR(diffv.w));
                    tmp.push_back(npnbor(diffv, dd));
                  }
                }
                if (tmp.size() > KNNOrder) {
                  nth_element(tmp.begin(), tmp.begin() + KNNOrder, tmp.end(), SortNPNeighborsForAscDistance);
                  mP[t].add(tmp[KNNOrder]);
                }
              }
              break;
            }
          }
        }
        // counting sort by type (:3975-3997)
        vector<size_t> s(MaxTypes, 0), e(MaxTypes, 0), c(MaxTypes, 0);
        for (auto& q : nb) c[q.m]++;
        size_t acc = 0;
        for (unsigned int ty = 0; ty < MaxTypes; ++ty) { s[ty] = acc; acc += c[ty]; e[ty] = acc; c[ty] = 0; }
        vector<apt_xyz> od(nb.size(), F32MX);
        for (auto& q : nb) { od.at(s[q.m] + c[q.m]) = q.d; c[q.m]++; }
        for (size_t t = 0; t < ntsk; ++t) {
          bool mine = false;
          for (auto& kt : tasks[t].trgcandidates) if (me.m == kt.second) { mine = true; break; }
          if (!mine) continue;
          auto& env = tasks[t].envcandidates;
          if (Settings::SpatStatDoRDF) for (auto& jt : env) for (size_t k = s[jt.second]; k < e[jt.second]; ++k) mR[t].add(od[k]);
          if (Settings::SpatStatDo1NN) {
            apt_real closest = F32MX; size_t id = SIZETMX;
            for (auto& jt : env) for (size_t k = s[jt.second]; k < e[jt.second]; ++k) {
              if (od[k] > closest) continue;
              closest = od[k]; id = k;
            }
            if (id != SIZETMX) m1[t].add(closest); else m1[t].add(R + EPSILON);
          }
          if (Settings::SpatStatDoRIPK) for (auto& jt : env) for (size_t k = s[jt.second]; k < e[jt.second]; ++k) mK[t].add(od[k]);
          if (Settings::SpatStatDoCountNbors) for (auto& jt : env) mC[t].add(e[jt.second] - s[jt.second], 1.f);
          if (Settings::SpatStatDoMKNN && !kcand.empty()) {
            vector<apt_xyz> tmp;
            for (auto& jt : env) for (size_t k = s[jt.second]; k < e[jt.second]; ++k) tmp.push_back(od[k]);
            for (size_t kth = 0; kth < kcand.size(); ++kth) {
              size_t ord = kcand[kth];
              size_t h = t * kcand.size() + kth;
              if (tmp.size() > ord) {
                nth_element(tmp.begin(), tmp.begin() + ord, tmp.end());
                mM[h].add(tmp[ord]);
              } else {
                mM[h].add(R + EPSILON);
              }
            }
          }
        }
      }
#pragma omp barrier
    }
#pragma omp critical
    {
      auto merge = [](histogram& g, histogram& m) {
        g.cnts_lowest += m.cnts_lowest;
        for (size_t b = 0; b < m.bincount(); ++b) g.cnts.at(b) += m.cnts.at(b);
        g.cnts_highest += m.cnts_highest;
      };
      for (size_t t = 0; t < ntsk; ++t) {
        if (Settings::SpatStatDoRDF) merge(gR[t], mR[t]);
        if (Settings::SpatStatDo1NN) merge(g1[t], m1[t]);
        if (Settings::SpatStatDoRIPK) merge(gK[t], mK[t]);
        if (Settings::SpatStatDoCountNbors) for (size_t b = 0; b < mC[t].cnts.size(); ++b) gC[t].add(b, mC[t].cnts.at(b));
      }
      for (size_t h = 0; h < mM.size(); ++h) merge(gM[h], mM[h]);
      for (size_t t = 0; t < mP.size(); ++t)
        for (size_t v = 0; v < mP[t].cnts.size(); ++v) gP[t].cnts[v] += mP[t].cnts[v];
    }
  }

  // ---- outputs
  auto names = [&](size_t t, string& a, string& b) { a = task_names(tasks[t].trgcandidates); b = task_names(tasks[t].envcandidates); };
  for (size_t t = 0; t < ntsk; ++t) {
    string a, b; names(t, a, b);
    if (Settings::SpatStatDoRDF) report2(outdir, E_RDF, "RDF", a, b, gR[t], rnd, nions_inside, volume_inside);
    if (Settings::SpatStatDo1NN) report2(outdir, E_NEAREST_NEIGHBOR, "1NN", a, b, g1[t], rnd, nions_inside, volume_inside);
    if (Settings::SpatStatDoRIPK) report2(outdir, E_RIPLEYK, "RIPK", a, b, gK[t], rnd, nions_inside, volume_inside);
  }
  for (size_t t = 0; t < ntsk; ++t) {
    string a, b; names(t, a, b);
    for (size_t kth = 0; kth < kcand.size(); ++kth)
      report2(outdir, E_MKNN, "MKNN" + to_string(kcand[kth] + 1), a, b, gM[t * kcand.size() + kth], rnd, nions_inside, volume_inside);
  }
  if (Settings::SpatStatDoCountNbors)
    for (size_t t = 0; t < ntsk; ++t) { string a, b; names(t, a, b); report3(outdir, a, b, gC[t], rnd); }

  vector<uint64_t> bins;
  auto put = [&](histogram& h) {
    bins.push_back((uint64_t)h.cnts_lowest);
    for (size_t b = 0; b < h.bincount(); ++b) bins.push_back((uint64_t)h.cnts[b]);
    bins.push_back((uint64_t)h.cnts_highest);
  };
  for (auto& h : gR) put(h);
  for (auto& h : g1) put(h);
  for (auto& h : gK) put(h);
  for (auto& h : gM) put(h);
  FILE* f = fopen((outdir + "/raw_bins.u64").c_str(), "wb");
  fwrite(bins.data(), 8, bins.size(), f);
  fclose(f);
  size_t L = 0;
  for (auto& h : gC) L = max(L, h.cnts.size());
  vector<uint64_t> cn;
  for (auto& h : gC) for (size_t b = 0; b < L; ++b) cn.push_back(b < h.cnts.size() ? (uint64_t)h.cnts[b] : 0);
  f = fopen((outdir + "/raw_cntnb.u64").c_str(), "wb");
  if (!cn.empty()) fwrite(cn.data(), 8, cn.size(), f);
  fclose(f);
  if (doP) {
    FILE* fp = fopen((outdir + "/raw_npcorr.u32").c_str(), "wb");
    for (auto& g : gP) fwrite(g.cnts.data(), 4, g.cnts.size(), fp);
    fclose(fp);
  }
  unsigned int nbins = histogram(Rs, Ri, Rm).bincount();
  ofstream st((outdir + "/stats.txt").c_str());
  st << "centres " << centres << "\ndiscarded " << discarded << "\npairs " << pairs << "\nnbins " << nbins
     << "\nntasks " << ntsk << "\nnk " << kcand.size() << "\ncntnb_len " << L << "\nmaxtypeid " << MaxTypes
     << "\nnpc_edge " << (doP ? npc3d(Rm, Ri, 0.f, false).get_support().nx : 0) << "\n";
  for (size_t t = 0; t < ntsk; ++t) {
    string a, b; names(t, a, b);
    st << "task " << t << " " << a << " " << b;
    for (auto& kv : tasks[t].trgcandidates) st << " T" << kv.second;
    for (auto& kv : tasks[t].envcandidates) st << " E" << kv.second;
    st << "\n";
  }
  for (size_t kth = 0; kth < kcand.size(); ++kth) st << "k " << kcand[kth] + 1 << "\n";
  return 0;
}
