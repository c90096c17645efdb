// pp_io.h -- host side of the drop-in: the inputs and outputs PARAPROBE's
// descriptive-statistics task reads and writes, restated in C++ above the
// C ABI of include/paraprobe_gb300.h.
//
//   Settings      XML keys of the spatial-statistics task
//                 (src/PARAPROBE_Settings.cpp:181-503, checks :871-905)
//   Ranging       RRNG range file -> ion types, m/q -> type
//                 (src/PARAPROBE_PeriodicTable.cpp:65-180, :324-420)
//   Task          "A,B-C,D;E-F" task codes
//                 (src/PARAPROBE_PeriodicTable.cpp:498-690)
//   POS / VTK     ion and hull readers
//                 (src/PARAPROBE_SolverHdl.cpp:6797-6930, :2029-2118)
//   CSV reports   RDF / 1NN / RIPK / MKNN / NBCNT files
//                 (src/PARAPROBE_SolverHdl.cpp:4299-4454)
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace ppio {

struct Settings {
  unsigned int sim_id = 0;
  int input_format = 0;          // 1 = POS
  std::string raw_file, rrng_file, surface_file;
  int recon_algo = 4;            // unknown values map to 4 (Bas et al.), as the reference does
  bool identify_ion_type = false;
  int surface_mode = 0;          // 4 = read an existing VTK hull
  bool debug_compute_distance = false;
  bool spatstat = false;         // any spatial-statistics analysis requested
  bool do_rdf = false, do_1nn = false, do_ripk = false, do_mknn = false, do_npcorr = false, do_cntnb = false;
  std::string tasks_code, mknn_code;
  float rmin = 0.f, rincr = 0.1f, rmax = 2.f;  // defaults of src/PARAPROBE_Settings.cpp:106-108
  size_t knn_order = 0;          // SpatStatKNNOrder - 1
  bool label_rnd = false;
  float carving_radius = 2.f;    // SurfaceCellsCarvingRadius default
  // occupancy-grid bin width keys (src/PARAPROBE_Settings.cpp:83-85, 460-465);
  // the grid behind the RDF header uses 0.5 (min + max)
  float bin_w_min = 1.f, bin_w_incr = 1.f, bin_w_max = 1.f;
  unsigned int rnd_seed = 0xffffffffu;
};

// Parse the XML file; throws std::runtime_error with the reason on failure.
Settings read_settings(const std::string& path);
// The validity checks of the spatial-statistics keys; empty string = valid.
std::string check_settings(const Settings& s);
// MKNN orders parsed from SpatStatMKNNCode, 1-based, sorted descending
// (src/PARAPROBE_SolverHdl.cpp:3739-3763).  Empty if the code holds a '-'.
std::vector<uint32_t> mknn_orders(const std::string& code);

struct MQRange { float lo, hi; };

struct Ranging {
  std::map<std::string, unsigned int> types;   // ion name -> type id (0 = "Unknown")
  std::vector<std::string> names;              // type id -> name
  std::vector<std::vector<MQRange>> ranges;    // type id -> ranges (sorted)
  unsigned int max_type_id() const { return (unsigned int)types.size(); }
  unsigned int type_of(float mq) const;
  // ranges flattened in the order type_of visits them (for device ranging)
  void flat(std::vector<float>& lo, std::vector<float>& hi, std::vector<uint8_t>& type) const;
};

// Returns false if the file cannot be opened (every ion stays type 0).
bool read_rrng(const std::string& path, Ranging& out);

struct Task {
  std::map<std::string, unsigned int> trg, env;
  std::string trg_name() const;
  std::string env_name() const;
};

std::vector<Task> parse_tasks(const std::string& code, const Ranging& rng);

bool read_pos(const std::string& path, std::vector<float>& xyz, std::vector<float>& mq);
// An EPOS file (src/PARAPROBE_SolverHdl.cpp:6933-7040, EPOS record of
// src/PARAPROBE_EPOSEndianness.h:87-140: 44-byte big-endian records of nine
// floats x, y, z, m/q, tof, Vdc, Vpulse, detx, dety and two int32 pulse
// fields) as the POS image of its reconstructed positions: per ion the first
// 16 bytes (x, y, z, m/q), the coordinates ReconstructionAlgorithm 3 takes
// as they are.  False if the file cannot be read or its size is not a
// multiple of 44 bytes.
bool read_epos_as_pos(const std::string& path, std::vector<uint8_t>& pos_image);
bool read_vtk_hull(const std::string& path, std::vector<float>& tri);

// One histogram as the reference holds it: counts per bin plus the dumps.
struct Histogram {
  double start, width;
  uint32_t nbins;
  std::vector<uint64_t> counts;  // nbins + 2: [lowest, bins..., highest]
};

enum class Report { RDF, NN1, RIPK, MKNN };

// Writes one file PARAPROBE.SimID.<id>.<metric>.<trg>.<env>.<Original|Rndmized>.csv
bool write_report(const std::string& dir, unsigned int sim_id, Report kind, const std::string& metric,
                  const std::string& trg, const std::string& env, const Histogram& h, bool randomized,
                  uint64_t nions_inside, double volume_inside);
bool write_nbcnt(const std::string& dir, unsigned int sim_id, const std::string& trg, const std::string& env,
                 const std::vector<uint64_t>& counts, bool randomized);

}  // namespace ppio
