// cru3d_main.cpp — drop-in replacement of the reference CLI (cpu/main.cpp),
// built on the C ABI only.
//
//   cru3d -param P.xml -mesh base [-out dir] [-start i] [-rank r]
//         [-engine plain|resident] [-precision 32|64]
//
// The reference runs sims_per_proc realizations one after another on one
// core (cpu/main.cpp:209-258); here they run as one batch on the GPU.  The
// per-realization seed follows cpu/RunSimulation.cpp:446 (93843 + seed_base +
// rank*seed_A + index*seed_B, plus the clock when flag_use_clock) and keys
// the Philox stream of that realization.  Outputs keep the reference names
// and formats: <out>/states_<rank>_<index>.out (float32 rows, see
// cpu/OutputFuncs.cpp:223-350) and grid_<rank>_<index>_<n>.vtk snapshots at
// the start, at every grid-output interval while it runs, and at its end.
#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "srs_gb300.h"

// Grid files during the run (cpu/RunSimulation.cpp:545-549): one per
// running realization at every grid-file step, numbered as the reference's
// output_counter.
struct GridOut {
  srs_sim* s;
  std::string out;
  int rank, idx0;
  std::vector<int> last;  // index of the last grid file written per realization
};
static void grid_cb(void* user, int64_t n, double t, const int* done) {
  GridOut* g = static_cast<GridOut*>(user);
  for (size_t i = 0; i < g->last.size(); ++i) {
    if (done[i]) continue;
    char fn[1024];
    std::snprintf(fn, sizeof(fn), "%s/grid_%d_%d_%d.vtk", g->out.c_str(), g->rank, g->idx0 + (int)i, (int)n);
    srs_write_grid_vtk(g->s, (int)i, fn, g->idx0 + (int)i, g->rank, (int)n, t);
    g->last[i] = (int)n;
  }
}

static int die(const char* what, int rc) {
  std::fprintf(stderr, "Error: %s: %s (%s)\n", what, srs_status_string(rc), srs_last_error());
  return 1;
}

int main(int argc, char** argv) {
  const char* param_file = "TestSet.xml";
  const char* out_dir = nullptr;
  const char* mesh_base = nullptr;
  int rank = 0, idx0 = 0, engine = SRS_ENGINE_RESIDENT, precision = SRS_FP32;
  for (int i = 1; i < argc; i += 2) {
    if (i + 1 >= argc) {
      std::fprintf(stderr, "Error: option %s needs a value\n", argv[i]);
      return 1;
    }
    if (!std::strcmp(argv[i], "-rank")) rank = std::atoi(argv[i + 1]);
    else if (!std::strcmp(argv[i], "-start")) idx0 = std::atoi(argv[i + 1]);
    else if (!std::strcmp(argv[i], "-param")) param_file = argv[i + 1];
    else if (!std::strcmp(argv[i], "-out")) out_dir = argv[i + 1];
    else if (!std::strcmp(argv[i], "-mesh")) mesh_base = argv[i + 1];
    else if (!std::strcmp(argv[i], "-engine"))
      engine = !std::strcmp(argv[i + 1], "plain") ? SRS_ENGINE_PLAIN : SRS_ENGINE_RESIDENT;
    else if (!std::strcmp(argv[i], "-precision")) precision = std::atoi(argv[i + 1]);
    else {
      std::fprintf(stderr, "Error: unrecognized command line option: %s\n", argv[i]);
      return 1;
    }
  }
  if (precision == SRS_FP64) engine = SRS_ENGINE_PLAIN;
  srs_params ps;
  srs_default_parameters(&ps);
  int rc = srs_read_parameters(&ps, param_file);
  if (rc) return die("reading parameters", rc);
  if (mesh_base) std::snprintf(ps.chars[0], 255, "%s", mesh_base);
  std::string out;
  if (out_dir) {
    out = out_dir;
  } else {
    char id[64];
    std::snprintf(id, sizeof(id), "%ld_%d", (long)std::time(nullptr), std::rand() % 1000);
    out = std::string("output/") + ps.chars[3] + "_" + id;
    mkdir("output", S_IRWXU);
  }
  mkdir(out.c_str(), S_IRWXU);
  std::printf("Output will be written to %s\n", out.c_str());
  srs_grid* g = nullptr;
  rc = srs_read_grid(&ps, ps.chars[0], &g);
  if (rc) return die("reading mesh", rc);
  srs_grid_info info;
  srs_grid_get_info(g, &info);
  std::printf("Done reading input mesh. # Faces = %d, # Elements = %d\n", info.n_face, info.n_ele);
  const int n_sims = ps.ints[17] - idx0;
  if (n_sims <= 0) {
    std::printf("Nothing to run (start index %d, sims_per_proc %d).\n", idx0, ps.ints[17]);
    srs_free_grid(g);
    return 0;
  }
  std::vector<uint64_t> seeds(n_sims);
  for (int i = 0; i < n_sims; ++i) {
    long long sd = 93843LL + ps.ints[3] + (long long)rank * ps.ints[4] + (long long)(idx0 + i) * ps.ints[5];
    if (ps.ints[2]) sd += (long long)std::time(nullptr);
    seeds[i] = (uint64_t)sd;
  }
  srs_sim_desc d;
  std::memset(&d, 0, sizeof(d));
  d.n_realizations = n_sims;
  d.precision = precision;
  d.engine = engine;
  d.seeds = seeds.data();
  srs_sim* s = nullptr;
  rc = srs_sim_create(g, &ps, &d, &s);
  if (rc) return die("creating simulation", rc);
  for (int i = 0; i < n_sims; ++i) {
    char fn[1024];
    std::snprintf(fn, sizeof(fn), "%s/grid_%d_%d_%d.vtk", out.c_str(), rank, idx0 + i, 0);
    if (ps.ints[0] || (rank == 0 && idx0 + i == 0)) srs_write_grid_vtk(s, i, fn, idx0 + i, rank, 0, 0.0);
  }
  // rows: t = 0, one per states interval, final
  double T = ps.reals[0], I = ps.reals[2];
  int64_t cap = (int64_t)(T / I) + 8;
  int width = SRS_STATES_ROW_BASE + (ps.ints[16] ? info.n_ryr : 0);
  std::vector<float> rows((size_t)n_sims * cap * width);
  std::vector<int64_t> n_rows(n_sims), n_steps(n_sims);
  std::vector<double> t_end(n_sims);
  srs_run_output ro{rows.data(), cap, width, n_rows.data(), t_end.data(), n_steps.data()};
  GridOut go{s, out, rank, idx0, std::vector<int>(n_sims, 0)};
  std::clock_t c0 = std::clock();
  rc = srs_run_simulation_grid(s, &ro, ps.ints[0] ? grid_cb : nullptr, &go, nullptr, 0, nullptr);
  std::clock_t c1 = std::clock();
  if (rc) return die("running simulation", rc);
  for (int i = 0; i < n_sims; ++i) {
    char fn[1024];
    std::snprintf(fn, sizeof(fn), "%s/states_%d_%d.out", out.c_str(), rank, idx0 + i);
    FILE* f = std::fopen(fn, "ab");
    if (!f) {
      std::fprintf(stderr, "Error opening states file %s\n", fn);
      return 1;
    }
    std::fwrite(&rows[(size_t)i * cap * width], sizeof(float), (size_t)n_rows[i] * width, f);
    std::fclose(f);
    // the final file takes the next index (cpu/RunSimulation.cpp:582)
    const int nf = go.last[i] + 1;
    std::snprintf(fn, sizeof(fn), "%s/grid_%d_%d_%d.vtk", out.c_str(), rank, idx0 + i, nf);
    if (ps.ints[0]) srs_write_grid_vtk(s, i, fn, idx0 + i, rank, nf, t_end[i]);
  }
  std::printf("Simulation completed in %f secs (rank %d, %d realizations).\n",
              (double)(c1 - c0) / CLOCKS_PER_SEC, rank, n_sims);
  srs_sim_destroy(s);
  srs_free_grid(g);
  return 0;
}
