// meshgen_main.cpp — writes a synthetic box-dyad mesh in the reference's
// mesh file set (see meshgen.cpp for the geometry).
//
//   srs_meshgen -out base [key value ...]
// keys: box_x box_y box_z foot_half_x foot_half_y n_foot_x n_foot_y n_out_x
//       n_out_y cleft_h jsr_h n_cleft_z n_jsr_z n_above_z r_trpn ryr_mode
//       ryr_nx ryr_ny ryr_pitch ryr_count ryr_radius n_lcc lcc_half lcc_seed seed
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "srs_gb300.h"

int main(int argc, char** argv) {
  srs_box_mesh_spec s;
  srs_box_mesh_default(&s);
  const char* out = nullptr;
  for (int i = 1; i + 1 < argc; i += 2) {
    const char* k = argv[i];
    const char* v = argv[i + 1];
    double x = std::atof(v);
    int n = std::atoi(v);
    if (!std::strcmp(k, "-out")) out = v;
    else if (!std::strcmp(k, "box_x")) s.box_x = x;
    else if (!std::strcmp(k, "box_y")) s.box_y = x;
    else if (!std::strcmp(k, "box_z")) s.box_z = x;
    else if (!std::strcmp(k, "foot_half_x")) s.foot_half_x = x;
    else if (!std::strcmp(k, "foot_half_y")) s.foot_half_y = x;
    else if (!std::strcmp(k, "n_foot_x")) s.n_foot_x = n;
    else if (!std::strcmp(k, "n_foot_y")) s.n_foot_y = n;
    else if (!std::strcmp(k, "n_out_x")) s.n_out_x = n;
    else if (!std::strcmp(k, "n_out_y")) s.n_out_y = n;
    else if (!std::strcmp(k, "cleft_h")) s.cleft_h = x;
    else if (!std::strcmp(k, "jsr_h")) s.jsr_h = x;
    else if (!std::strcmp(k, "n_cleft_z")) s.n_cleft_z = n;
    else if (!std::strcmp(k, "n_jsr_z")) s.n_jsr_z = n;
    else if (!std::strcmp(k, "n_above_z")) s.n_above_z = n;
    else if (!std::strcmp(k, "r_trpn")) s.r_trpn = x;
    else if (!std::strcmp(k, "ryr_mode")) s.ryr_mode = n;
    else if (!std::strcmp(k, "ryr_nx")) s.ryr_nx = n;
    else if (!std::strcmp(k, "ryr_ny")) s.ryr_ny = n;
    else if (!std::strcmp(k, "ryr_pitch")) s.ryr_pitch = x;
    else if (!std::strcmp(k, "ryr_count")) s.ryr_count = n;
    else if (!std::strcmp(k, "ryr_radius")) s.ryr_radius = x;
    else if (!std::strcmp(k, "n_lcc")) s.n_lcc = n;
    else if (!std::strcmp(k, "lcc_half")) s.lcc_half = x;
    else if (!std::strcmp(k, "lcc_seed")) s.lcc_seed = (uint64_t)std::strtoull(v, nullptr, 10);
    else if (!std::strcmp(k, "seed")) s.seed = (uint64_t)std::strtoull(v, nullptr, 10);
    else {
      std::fprintf(stderr, "unknown key %s\n", k);
      return 1;
    }
  }
  if (!out) {
    std::fprintf(stderr, "usage: srs_meshgen -out base [key value ...]\n");
    return 1;
  }
  int rep[6];
  double a0;
  int rc = srs_box_mesh_write(&s, out, rep, &a0);
  if (rc) {
    std::fprintf(stderr, "Error: %s (%s)\n", srs_status_string(rc), srs_last_error());
    return 1;
  }
  std::printf("tets %d faces %d nodes %d ryr %d lcc %d jsr_tets %d max_a0 %.6g\n", rep[0], rep[1],
              rep[2], rep[3], rep[4], rep[5], a0);
  return 0;
}
