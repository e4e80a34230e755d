// meshgen_main.cpp — writes a synthetic box-dyad mesh in the reference's
// mesh file set (see meshgen.cpp for the geometry).  Host code only: it is
// built from meshgen.cpp alone and loads no CUDA library, so CPU-only
// callers (the CPU reference timings) can write their inputs with it.
//
//   srs_meshgen -out base [key value ...]
// keys: box_x box_y box_z foot_half_x foot_half_y n_foot_x n_foot_y n_out_x
//       n_out_y cleft_h jsr_h n_cleft_z n_jsr_z n_above_z r_trpn ryr_mode
//       ryr_nx ryr_ny ryr_pitch ryr_count ryr_radius n_lcc lcc_half lcc_seed seed
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "srs_host.h"

int main(int argc, char** argv) {
  srs::MeshGenSpec s;
  srs::meshgen_default_spec(&s);
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
  srs::MeshGenReport rep;
  int rc = srs::meshgen_box(s, out, &rep);
  if (rc) {
    std::fprintf(stderr, "Error: mesh generation failed (status %d) for %s\n", rc, out);
    return 1;
  }
  std::printf("tets %d faces %d nodes %d ryr %d lcc %d jsr_tets %d max_a0 %.6g\n", rep.n_tets,
              rep.n_faces, rep.n_nodes, rep.n_ryr, rep.n_lcc, rep.n_jsr_tets, rep.max_a0);
  return 0;
}
