// pp_io.cpp -- settings, ranging, task parsing, readers and CSV writers of the
// descriptive-statistics task, restated in C++ for the GB300 drop-in.
#include "pp_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>

namespace ppio {

namespace {

constexpr double kEpsilon = 1.0e-6;  // src/PARAPROBE_Numerics.h:44
// src/PARAPROBE_Abinitio.h:38
constexpr double kPi = 3.141592653589793238462643383279502884197169399375105820974;

// ------------------------------------------------------------------ XML
// The settings file is a flat <Parameters> element with one child element per
// key.  Only direct children of the root are looked up, by name, first match
// (as rapidxml's first_node does); the value is the element's text with the
// five predefined entities translated.
struct Xml {
  std::string root;
  std::map<std::string, std::string> first;
};

std::string unescape(const std::string& s) {
  std::string o;
  for (size_t i = 0; i < s.size(); ++i) {
    if (s[i] == '&') {
      static const char* ent[][2] = {{"&lt;", "<"}, {"&gt;", ">"}, {"&amp;", "&"}, {"&quot;", "\""}, {"&apos;", "'"}};
      bool hit = false;
      for (auto& e : ent) {
        const size_t L = std::strlen(e[0]);
        if (s.compare(i, L, e[0]) == 0) { o += e[1]; i += L - 1; hit = true; break; }
      }
      if (!hit) o += s[i];
    } else {
      o += s[i];
    }
  }
  return o;
}

Xml parse_xml(const std::string& doc) {
  Xml x;
  size_t i = 0;
  int depth = 0;
  std::vector<std::string> stack;
  std::string pending_name;
  size_t text_begin = std::string::npos;
  while (i < doc.size()) {
    if (doc[i] != '<') { ++i; continue; }
    if (doc.compare(i, 4, "<!--") == 0) {
      const size_t e = doc.find("-->", i + 4);
      if (e == std::string::npos) throw std::runtime_error("unterminated XML comment");
      i = e + 3;
      continue;
    }
    if (doc.compare(i, 2, "<?") == 0) {
      const size_t e = doc.find("?>", i + 2);
      if (e == std::string::npos) throw std::runtime_error("unterminated XML declaration");
      i = e + 2;
      continue;
    }
    if (doc.compare(i, 2, "<!") == 0) {
      const size_t e = doc.find('>', i + 2);
      if (e == std::string::npos) throw std::runtime_error("unterminated XML markup");
      i = e + 1;
      continue;
    }
    const size_t e = doc.find('>', i);
    if (e == std::string::npos) throw std::runtime_error("unterminated XML tag");
    std::string tag = doc.substr(i + 1, e - i - 1);
    const bool closing = !tag.empty() && tag[0] == '/';
    const bool selfclose = !tag.empty() && tag.back() == '/';
    std::string name = closing ? tag.substr(1) : (selfclose ? tag.substr(0, tag.size() - 1) : tag);
    name = name.substr(0, name.find_first_of(" \t\r\n"));
    if (closing) {
      if (stack.empty() || stack.back() != name) throw std::runtime_error("mismatched XML tag </" + name + ">");
      if (depth == 2 && text_begin != std::string::npos && !x.first.count(name))
        x.first[name] = unescape(doc.substr(text_begin, i - text_begin));
      stack.pop_back();
      --depth;
      text_begin = std::string::npos;
    } else {
      if (depth == 0) x.root = name;
      if (selfclose) {
        if (depth == 1 && !x.first.count(name)) x.first[name] = "";
      } else {
        stack.push_back(name);
        ++depth;
        text_begin = (depth == 2) ? e + 1 : std::string::npos;
      }
    }
    i = e + 1;
  }
  return x;
}

unsigned long to_ul(const std::string& s) { return std::stoul(s); }
float to_real(const std::string& s) { return std::stof(s); }  // str2real with single precision

}  // namespace

// src/PARAPROBE_Settings.cpp:181-503 (the keys this path reads)
Settings read_settings(const std::string& path) {
  std::ifstream f(path);
  if (f.fail()) throw std::runtime_error("Unable to locate input file " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const Xml x = parse_xml(ss.str());
  if (x.root != "Parameters") throw std::runtime_error("Undefined parameters file!");
  auto has = [&](const char* k) { return x.first.count(k) > 0; };
  auto val = [&](const char* k) { return x.first.at(k); };
  Settings s;
  unsigned long mode = 0;
  if (has("InputFileformat")) mode = to_ul(val("InputFileformat"));
  s.input_format = (mode >= 1 && mode <= 4) ? (int)mode : 0;
  if (has("RAWFilenameIn")) s.raw_file = val("RAWFilenameIn");
  mode = 4;
  if (has("ReconstructionAlgorithm")) mode = to_ul(val("ReconstructionAlgorithm"));
  s.recon_algo = (mode <= 4) ? (int)mode : 4;
  if (has("IdentifyIonType")) s.identify_ion_type = to_ul(val("IdentifyIonType")) != 0;
  if (has("RRNGFilenameIn")) s.rrng_file = val("RRNGFilenameIn");
  mode = 0;
  if (has("SurfaceReconstructionType")) mode = to_ul(val("SurfaceReconstructionType"));
  s.surface_mode = (mode <= 4) ? (int)mode : 0;
  if (has("SurfaceFilenameIn")) s.surface_file = val("SurfaceFilenameIn");
  // AnalysisSpatDistrType: one digit selects one analysis; several digits (at
  // most four, no zero) select several (src/PARAPROBE_Settings.cpp:348-392)
  bool any = false;
  if (has("AnalysisSpatDistrType")) {
    mode = to_ul(val("AnalysisSpatDistrType"));
    switch (mode) {
      case 1: s.do_rdf = any = true; break;
      case 2: s.do_1nn = any = true; break;
      case 3: s.do_ripk = any = true; break;
      case 4: s.do_mknn = any = true; break;
      case 5: s.do_npcorr = any = true; break;
      case 6: s.do_cntnb = any = true; break;
      default: {
        const std::string m = val("AnalysisSpatDistrType");
        if (m.find('0') != std::string::npos || m.size() > 4 || m.size() < 1) break;
        if (m.find('1') != std::string::npos) s.do_rdf = any = true;
        if (m.find('2') != std::string::npos) s.do_1nn = any = true;
        if (m.find('3') != std::string::npos) s.do_ripk = any = true;
        if (m.find('4') != std::string::npos) s.do_mknn = any = true;
        if (m.find('5') != std::string::npos) s.do_npcorr = any = true;
        if (m.find('6') != std::string::npos) s.do_cntnb = any = true;
      }
    }
  }
  s.spatstat = any;
  int tess = 0;
  if (has("AnalysisVolumeTessellation")) tess = to_ul(val("AnalysisVolumeTessellation")) == 1 ? 1 : 0;
  if (has("AdvIonPruneBinWidthMin")) s.bin_w_min = to_real(val("AdvIonPruneBinWidthMin"));
  if (has("AdvIonPruneBinWidthIncr")) s.bin_w_incr = to_real(val("AdvIonPruneBinWidthIncr"));
  if (has("AdvIonPruneBinWidthMax")) s.bin_w_max = to_real(val("AdvIonPruneBinWidthMax"));
  if (has("DebugComputeDistance")) s.debug_compute_distance = to_ul(val("DebugComputeDistance")) == 1;
  if (s.spatstat) {
    if (has("DescrStatTasksCode")) s.tasks_code = val("DescrStatTasksCode");
    if (has("SpatStatRadiusMin")) s.rmin = to_real(val("SpatStatRadiusMin"));
    if (has("SpatStatRadiusIncr")) s.rincr = to_real(val("SpatStatRadiusIncr"));
    if (has("SpatStatRadiusMax")) s.rmax = to_real(val("SpatStatRadiusMax"));
    if (has("SpatStatKNNOrder")) {
      const unsigned long v = to_ul(val("SpatStatKNNOrder"));
      if (v > 0) s.knn_order = v - 1;
    }
    if (s.do_mknn && has("SpatStatMKNNCode")) s.mknn_code = val("SpatStatMKNNCode");
    if (has("SpatStatAdditionalLabelRandomization"))
      s.label_rnd = to_ul(val("SpatStatAdditionalLabelRandomization")) == 1;
  }
  if (tess && has("SurfaceCellsCarvingRadius")) s.carving_radius = to_real(val("SurfaceCellsCarvingRadius"));
  return s;
}

// src/PARAPROBE_Settings.cpp:645-905 (the checks that concern this path)
std::string check_settings(const Settings& s) {
  if (s.recon_algo == 2 && s.input_format != 1 && s.input_format != 3)
    return "ReconstructionAlgorithm is POS but InputFileformat is neither POS nor HDF5!";
  if (s.recon_algo == 3 && s.input_format != 2) return "ReconstructionAlgorithm is EPOS but InputFileformat is not EPOS!";
  if (s.recon_algo == 4 && s.input_format != 2) return "Reconstruction is Bas et al. but InputFileformat is not EPOS!";
  if (s.bin_w_min > s.bin_w_max || s.bin_w_min > s.bin_w_incr || s.bin_w_max < s.bin_w_incr)
    return "Invalid choice for AdvIonPruneBinning";
  if (s.spatstat) {
    if (s.rmin < 0.f) return "SpatStatRadiusMin must be positive or zero!";
    if (s.rincr < kEpsilon) return "SpatStatRadiusIncr must be positive!";
    if (s.rmax < kEpsilon) return "SpatStatRadiusMax must be positive!";
    if (s.rmin >= s.rmax) return "SpatStatRadiusMin is larger than SpatStatRadiusMax!";
  }
  return "";
}

std::vector<uint32_t> mknn_orders(const std::string& code) {
  std::vector<uint32_t> ks;
  if (code.empty() || code.find('-') != std::string::npos) return ks;
  const int nsemi = (int)std::count(code.begin(), code.end(), ';');
  std::istringstream line(code);
  std::string piece;
  for (int i = 0; i <= nsemi; ++i) {
    std::getline(line, piece, ';');
    const bool number = !piece.empty() && std::all_of(piece.begin(), piece.end(), [](char c) {
      return std::isdigit((unsigned char)c) != 0;
    });
    if (number) {
      const unsigned long v = std::stoul(piece);
      if (v < 1) throw std::runtime_error("Instructing a kth order value smaller than 1");
      ks.push_back((uint32_t)v);
    }
  }
  std::sort(ks.begin(), ks.end(), [](uint32_t a, uint32_t b) { return a > b; });
  return ks;
}

// ---------------------------------------------------------------- ranging
namespace {
// Chemical element symbols for Z = 1..92 and Pu: the keys an RRNG ion
// description is matched against (the same set PeriodicTable loads,
// src/PARAPROBE_PeriodicTable.cpp:696-800); kept in a sorted map so molecular
// ion names concatenate element symbols in lexicographic order.
const std::vector<std::string>& element_symbols() {
  static const std::vector<std::string> v = [] {
    const char* z[] = {
        "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",  "S",
        "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge",
        "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd",
        "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd",
        "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au", "Hg",
        "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U",  "Pu"};
    std::vector<std::string> s(std::begin(z), std::end(z));
    std::sort(s.begin(), s.end());
    return s;
  }();
  return v;
}

std::vector<std::string> split_any(const std::string& line, const char* delims) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : line) {
    if (std::strchr(delims, c)) { out.push_back(cur); cur.clear(); }
    else cur.push_back(c);
  }
  out.push_back(cur);
  return out;
}

// Ion name of one RRNG range line: every element symbol that occurs in a
// description token (tokens 3 .. n-2), single-letter symbols only as "X:"
// (src/PARAPROBE_PeriodicTable.cpp:119-153).
std::string ion_name(const std::vector<std::string>& tok) {
  std::string cand;
  for (const std::string& el : element_symbols()) {
    for (size_t k = 3; k + 1 < tok.size(); ++k) {
      const bool hit = el.size() == 1 ? tok[k].find(el + ":") != std::string::npos
                                      : tok[k].find(el) != std::string::npos;
      if (hit) { cand += el; break; }
    }
  }
  return cand;
}
}  // namespace

unsigned int Ranging::type_of(float mq) const {
  for (size_t t = 0; t < ranges.size(); ++t)
    for (const MQRange& r : ranges[t])
      if (!(mq < r.lo) && !(mq > r.hi)) return (unsigned int)t;
  return 0;
}

void Ranging::flat(std::vector<float>& lo, std::vector<float>& hi, std::vector<uint8_t>& type) const {
  lo.clear(); hi.clear(); type.clear();
  for (size_t t = 0; t < ranges.size(); ++t)
    for (const MQRange& r : ranges[t]) { lo.push_back(r.lo); hi.push_back(r.hi); type.push_back((uint8_t)t); }
}

// src/PARAPROBE_PeriodicTable.cpp:324-420: skip to "[Ranges]", then every line
// "RangeN=lo hi Vol:... El:n ... Color:..." adds [lo, hi] to its ion type;
// types are numbered in order of first appearance after "Unknown" = 0.
bool read_rrng(const std::string& path, Ranging& out) {
  out = Ranging();
  out.types["Unknown"] = 0;
  out.names.push_back("Unknown");
  out.ranges.push_back({MQRange{0.0f, 0.001f}});
  std::ifstream f(path);
  if (!f.is_open()) return false;
  std::string line;
  while (f.good()) {
    std::getline(f, line);
    if (line.find("[Ranges]") != std::string::npos) break;
  }
  while (f.good()) {
    std::getline(f, line);
    const std::vector<std::string> tok = split_any(line, " \t");
    if (tok.size() >= 5 && tok[0].find("Range") != std::string::npos && tok[2].find("Vol") != std::string::npos) {
      std::istringstream ls(line);
      std::string piece;
      std::getline(ls, piece, '=');
      std::getline(ls, piece, ' ');
      const float lo = std::stof(piece);
      std::getline(ls, piece, ' ');
      const float hi = std::stof(piece);
      const std::string name = ion_name(tok);
      auto it = out.types.find(name);
      if (it == out.types.end()) {
        const unsigned int id = (unsigned int)out.types.size();
        out.types[name] = id;
        out.names.push_back(name);
        out.ranges.push_back({MQRange{lo, hi}});
      } else {
        out.ranges[it->second].push_back(MQRange{lo, hi});
      }
    }
  }
  for (auto& r : out.ranges)
    std::sort(r.begin(), r.end(), [](const MQRange& a, const MQRange& b) { return a.hi < b.lo; });
  return true;
}

// ------------------------------------------------------------------ tasks
std::string Task::trg_name() const {
  std::string s;
  for (auto& kv : trg) s += kv.first;
  return s;
}
std::string Task::env_name() const {
  std::string s;
  for (auto& kv : env) s += kv.first;
  return s;
}

namespace {
// A user-written ion name -> the internal name: the element symbols it
// contains, taken in lexicographic order, unless it is exactly one symbol
// (src/PARAPROBE_PeriodicTable.cpp:546-583).
std::string canonical(const std::string& piece) {
  std::vector<std::string> found;
  for (const std::string& el : element_symbols())
    if (piece.find(el) != std::string::npos) found.push_back(el);
  for (const std::string& el : found)
    if (piece == el) return el;
  std::string c;
  for (const std::string& el : found) c += el;
  return c;
}

void fill(const std::string& part, const Ranging& rng, std::map<std::string, unsigned int>& into) {
  const size_t n = (size_t)std::count(part.begin(), part.end(), ',') + 1;
  std::istringstream ss(part);
  std::string piece;
  for (size_t i = 0; i < n; ++i) {
    std::getline(ss, piece, ',');
    const std::string c = canonical(piece);
    auto it = rng.types.find(c);
    if (it != rng.types.end()) into.insert(*it);
  }
}
}  // namespace

// src/PARAPROBE_PeriodicTable.cpp:498-690: ';' separates tasks, one '-'
// separates centres from environment, ',' separates ion names; tasks with an
// empty centre or environment set are dropped.
std::vector<Task> parse_tasks(const std::string& code, const Ranging& rng) {
  std::vector<Task> tasks;
  if (code.empty()) return tasks;
  const int n = (int)std::count(code.begin(), code.end(), ';') + 1;
  std::stringstream ss;
  ss << code;
  std::string piece;
  for (int t = 0; t < n; ++t) {
    std::getline(ss, piece, ';');
    if (piece.empty() || std::count(piece.begin(), piece.end(), '-') != 1) continue;
    std::istringstream line(piece);
    std::string centers, nbors;
    std::getline(line, centers, '-');
    std::getline(line, nbors, '-');
    Task task;
    fill(centers, rng, task.trg);
    if (task.trg.empty()) continue;
    fill(nbors, rng, task.env);
    if (task.env.empty()) continue;
    tasks.push_back(task);
  }
  return tasks;
}

// ---------------------------------------------------------------- readers
bool read_epos_as_pos(const std::string& path, std::vector<uint8_t>& pos_image) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0 || sz % 44) { std::fclose(f); return false; }
  const size_t n = (size_t)sz / 44;
  std::vector<uint8_t> raw((size_t)sz);
  const size_t got = std::fread(raw.data(), 1, raw.size(), f);
  std::fclose(f);
  if (got != raw.size()) return false;
  pos_image.resize(16 * n);
  for (size_t i = 0; i < n; ++i) std::memcpy(&pos_image[16 * i], &raw[44 * i], 16);
  return true;
}

bool read_pos(const std::string& path, std::vector<float>& xyz, std::vector<float>& mq) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0 || sz % 16) { std::fclose(f); return false; }
  const size_t n = (size_t)sz / 16;
  std::vector<uint8_t> raw((size_t)sz);
  const size_t got = std::fread(raw.data(), 1, raw.size(), f);
  std::fclose(f);
  if (got != raw.size()) return false;
  xyz.resize(3 * n);
  mq.resize(n);
  auto be = [&](size_t off) {
    const uint32_t u = ((uint32_t)raw[off] << 24) | ((uint32_t)raw[off + 1] << 16) | ((uint32_t)raw[off + 2] << 8) |
                       (uint32_t)raw[off + 3];
    float v;
    std::memcpy(&v, &u, 4);
    return v;
  };
  for (size_t i = 0; i < n; ++i) {
    xyz[3 * i] = be(16 * i);
    xyz[3 * i + 1] = be(16 * i + 4);
    xyz[3 * i + 2] = be(16 * i + 8);
    mq[i] = be(16 * i + 12);
  }
  return true;
}

bool read_vtk_hull(const std::string& path, std::vector<float>& tri) {
  std::ifstream f(path);
  if (!f.is_open()) return false;
  std::string line, tok;
  for (int i = 0; i < 4; ++i) std::getline(f, line);
  std::getline(f, line);
  if (line.empty()) return false;
  std::istringstream ls(line);
  std::getline(ls, tok, ' ');
  std::getline(ls, tok, ' ');
  const size_t nv = std::stoul(tok);
  if (nv % 3) return false;
  tri.clear();
  tri.reserve(nv * 3);
  size_t v = 0;
  while (v < nv && f.good()) {
    for (int k = 0; k < 3; ++k) {
      std::getline(f, line);
      std::istringstream s(line);
      for (int q = 0; q < 3; ++q) {
        std::getline(s, tok, ' ');
        tri.push_back(std::stof(tok));
      }
    }
    v += 3;
  }
  return v == nv;
}

// ---------------------------------------------------------------- reports
namespace {
std::string report_name(const std::string& dir, unsigned int sim_id, const std::string& metric, const std::string& trg,
                        const std::string& env, bool randomized) {
  std::string fn = "PARAPROBE.SimID." + std::to_string(sim_id) + "." + metric + "." + trg + "." + env;
  fn += randomized ? ".Rndmized.csv" : ".Original.csv";
  return dir.empty() ? fn : dir + "/" + fn;
}
}  // namespace

// The file layouts of src/PARAPROBE_SolverHdl.cpp:4299-4410, printed with the
// same stream precision (18 significant digits) and the same double
// expressions, so the files are byte-identical for identical counts.
bool write_report(const std::string& dir, unsigned int sim_id, Report kind, const std::string& metric,
                  const std::string& trg, const std::string& env, const Histogram& h, bool randomized,
                  uint64_t nions_inside, double volume_inside) {
  std::ofstream o(report_name(dir, sim_id, metric, trg, env, randomized));
  if (!o.is_open()) return false;
  o.precision(18);
  const double start = h.start, width = h.width;
  auto count = [&](uint32_t b) { return (double)h.counts[1 + b]; };
  const double lowest = (double)h.counts[0], highest = (double)h.counts[h.nbins + 1];
  double bend = start + width;
  if (kind == Report::RDF) {
    o << "NumberOfIonsInside" << ";" << nions_inside << "\n";
    o << "VolumeInside" << ";" << volume_inside << " (nm^3)\n";
    if (volume_inside > kEpsilon) {
      double density = (double)nions_inside;
      density /= volume_inside;
      o << "InsideAtomicDensityEst" << ";" << density << "\n";
      const double norm = (1.f / density) * (1.f / ((4.f / 3.f) * kPi));
      o << "NormalizationFactor" << ";" << norm << "\n";
      o << "r;AccumulatedCount;nRDF(r);ShellVolume;RDF(r)\n";
      o << "nm;1;1;nm^3;1\n";
      o << "r;AccumulatedCount;nRDF(r);ShellVolume;RDF(r)\n";
      o << start << ";" << lowest << ";;;\n";
      const double half = 0.5 * width;
      for (uint32_t b = 0; b < h.nbins; ++b, bend += width) {
        const double r = start + (0.5 + (double)b) * width;
        const double diff = (b > 0) ? (count(b) - count(b - 1)) : 0.f;
        const double a = r + half, c = r - half;
        const double shell = a * a * a - c * c * c;
        const double rdf = (shell > kEpsilon) ? norm * diff / shell : 0.f;
        o << r << ";" << count(b) << ";" << diff << ";" << shell << ";" << rdf << "\n";
      }
      o << "" << ";" << highest << ";;;\n";
    }
  }
  if (kind == Report::NN1 || kind == Report::MKNN) {
    o << (kind == Report::NN1 ? std::string("1NN") : metric) << "\n";
    o << "BinEnd(r);Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
    o << "nm;1;1;1\n";
    o << "BinEnd(r);Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
    o << start << ";" << lowest << ";;\n";
    double total = 0.f;
    for (uint32_t b = 0; b < h.nbins; ++b) total += count(b);
    double sum = 0.f;
    for (uint32_t b = 0; b < h.nbins; ++b, bend += width) {
      sum += count(b);
      const double cdf = (total > kEpsilon) ? (sum / total) : 0.f;
      o << bend << ";" << count(b) << ";" << sum << ";" << cdf << "\n";
    }
    o << "" << ";" << highest << ";;\n";
  }
  if (kind == Report::RIPK) {
    o << "BinEnd(r);AccumulatedCounts\n";
    o << "nm;1\n";
    o << "BinEnd(r);AccumulatedCounts\n";
    o << start << ";" << lowest << "\n";
    double sum = 0;
    for (uint32_t b = 0; b < h.nbins; ++b, bend += width) {
      sum += count(b);
      o << bend << ";" << sum << "\n";
    }
    o << "" << ";" << highest << "\n";
  }
  return o.good();
}

// src/PARAPROBE_SolverHdl.cpp:4412-4454
bool write_nbcnt(const std::string& dir, unsigned int sim_id, const std::string& trg, const std::string& env,
                 const std::vector<uint64_t>& counts, bool randomized) {
  std::ofstream o(report_name(dir, sim_id, "NBCNTinRMAX", trg, env, randomized));
  if (!o.is_open()) return false;
  o.precision(18);
  o << "NeighborCountInRMax\n";
  o << "Value;Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
  o << "1;1;1;1\n";
  o << "Value;Counts;ECDFon[BinMinBinMax];CDFon[BinMinBinMax]\n";
  // the reference holds these counts in float (apt_real), which is exact
  // below 2^24 per bin
  double total = 0.f;
  for (uint64_t c : counts) total += (double)(float)c;
  double sum = 0.f;
  for (size_t b = 0; b < counts.size(); ++b) {
    const float c = (float)counts[b];
    sum += c;
    const double cdf = (total > kEpsilon) ? (sum / total) : 0.f;
    o << b << ";" << c << ";" << sum << ";" << cdf << "\n";
  }
  return o.good();
}

}  // namespace ppio
