// srs_host.cpp — parameter parsing, mesh loading, renumbering, operator
// assembly, initial state, step schedule and output formatting.
#include "srs_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <sstream>

namespace srs {

void diffusion_by_species(const srs_params& p, double D[N_SPECIES]) {
  // ps->Diff[] (cpu/InitFuncs.cpp:359-364)
  D[SP_CA] = p.reals[R_D_CA];
  D[SP_ATP] = p.reals[R_D_ATP];
  D[SP_CMDN] = p.reals[R_D_CMDN];
  D[SP_TRPN] = p.reals[R_D_TRPN];
  D[SP_CSQN] = p.reals[R_D_CSQN];
  D[SP_DYE] = p.reals[R_D_DYE];
}

void params_default(srs_params* p) {
  std::memset(p, 0, sizeof(*p));
  int* I = p->ints;
  double* R = p->reals;
  I[I_OUTPUT_GRID_FLAG] = 0;
  I[I_FLAG_FIDELITY_SIM] = 0;
  I[I_FLAG_CLOCK_SEED] = 1;
  I[I_RAND_SEED_0] = 38376427;
  I[I_RAND_ADD_A] = 12783;
  I[I_RAND_ADD_B] = 83;
  I[I_INITIALIZE_FROM_FILE] = 0;
  I[I_CUDA_DEVICE] = 0;
  I[I_FLAG_SECONDARY_GRADIENT] = 0;
  I[I_FLAG_NO_FLUX_BOUNDARY] = 1;
  I[I_N_RYR_FIDELITY] = 1000;
  I[I_FLAG_LCC] = 0;
  I[I_LCC_INDEX] = 0;
  I[I_FLAG_V_CLAMP] = 0;
  I[I_FLAG_NO_GATING] = 0;
  I[I_GATING_FFWD] = 0;
  I[I_FLAG_RYR_OUT] = 0;
  I[I_N_SIMS] = 1;
  I[I_INIT_RYR] = -1;
  R[R_T_FINAL] = 500;
  R[R_T_STEP] = 12e-6;
  R[R_OUTPUT_STATES_INTERVAL] = 0.01;
  R[R_OUTPUT_GRID_INTERVAL] = 1;
  R[R_C_MIN] = 1.0;
  R[R_D_CA] = 0.25;
  R[R_D_CA_JSR] = 0.25;
  R[R_D_ATP] = 0.14;
  R[R_D_CMDN] = 0.025;
  R[R_D_TRPN] = 0;
  R[R_D_CSQN] = 0;
  R[R_D_DYE] = 0.042;
  R[R_D_EGTA] = 0;
  R[R_C_0_CA] = 0.1;
  R[R_C_0_CA_JSR] = 1000;
  R[R_DEFAULT_VM] = -80;
  R[R_DEFAULT_CA_NSR] = 1000;
  R[R_CA_0] = 2000;
  R[R_B_TOT_ATP] = 455;
  R[R_K_OFF_ATP] = 45;
  R[R_K_ON_ATP] = 0.225;
  R[R_B_TOT_CMDN] = 24;
  R[R_K_OFF_CMDN] = 0.238;
  R[R_K_ON_CMDN] = 0.034;
  R[R_B_TOT_TRPN] = 70;
  R[R_K_OFF_TRPN] = 0.02;
  R[R_K_ON_TRPN] = 0.039;
  R[R_B_TOT_SL_HI] = 1.6e-13;
  R[R_K_D_SL_HI] = 13;
  R[R_B_TOT_SL_LO] = 0;
  R[R_K_D_SL_LO] = 1100;
  R[R_B_TOT_DYE] = 50;
  R[R_K_OFF_DYE] = 0.110;
  R[R_K_ON_DYE] = 0.10;
  R[R_B_T_JSR] = 30000;
  R[R_K_M_JSR] = 638;
  R[R_V_REFILL] = 0.095;
  R[R_V_RYR] = 3e-8;
  R[R_V_CELL] = 25.84e3;
  R[R_K_ON_CSQN] = 0.10;
  R[R_K_OFF_CSQN] = 63.8;
  R[R_RYR_ETA] = 2.1;
  R[R_RYR_A_STAR] = 0;
  R[R_RYR_EPS_CC] = -0.92;
  R[R_RYR_EPS_OO] = -0.85;
  R[R_RYR_K_PLUS] = 0.1107e-3;
  R[R_RYR_K_MINUS] = 0.500;
  R[R_RYR_PHI_M] = 4.0;
  R[R_RYR_PHI_B] = 1500;
  R[R_K_D_i] = 910;
  R[R_K_D_SR] = 2240;
  R[R_A_P] = 150;
  R[R_LCC_DURATION] = 0.5;
  R[R_T_CLAMP] = 200;
  R[R_V_CLAMP] = 0;
  R[R_INIT_RYR_HOLD] = 0;
  std::snprintf(p->chars[C_FILE_BASE], 255, "mesh");
  std::snprintf(p->chars[C_OUTPUT_STATE], 255, "output");
  std::snprintf(p->chars[C_OUTPUT_GRID], 255, "output");
  std::snprintf(p->chars[C_PARAM_TITLE], 255, "Untitled");
}

namespace {

std::string xml_decode(const std::string& s) {
  std::string o;
  o.reserve(s.size());
  for (size_t i = 0; i < s.size(); ++i) {
    if (s[i] != '&') {
      o += s[i];
      continue;
    }
    size_t e = s.find(';', i);
    if (e == std::string::npos) {
      o += s[i];
      continue;
    }
    std::string ent = s.substr(i + 1, e - i - 1);
    if (ent == "lt") o += '<';
    else if (ent == "gt") o += '>';
    else if (ent == "amp") o += '&';
    else if (ent == "quot") o += '"';
    else if (ent == "apos") o += '\'';
    else if (!ent.empty() && ent[0] == '#') {
      long c = (ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X'))
                   ? std::strtol(ent.c_str() + 2, nullptr, 16)
                   : std::strtol(ent.c_str() + 1, nullptr, 10);
      if (c > 0 && c < 128) o += (char)c;
    } else {
      o += s.substr(i, e - i + 1);
    }
    i = e;
  }
  return o;
}

// Text content of the first child element <tag> inside [b, e) of s.
bool child_text(const std::string& s, size_t b, size_t e, const char* tag, std::string* out) {
  std::string open = std::string("<") + tag;
  size_t p = b;
  while (true) {
    p = s.find(open, p);
    if (p == std::string::npos || p >= e) return false;
    char c = s[p + open.size()];
    if (c == '>' || c == '/' || c == ' ' || c == '\t' || c == '\n' || c == '\r') break;
    p += open.size();
  }
  size_t gt = s.find('>', p);
  if (gt == std::string::npos || gt >= e) return false;
  if (s[gt - 1] == '/') {  // <tag/>
    *out = "";
    return true;
  }
  std::string close = std::string("</") + tag + ">";
  size_t q = s.find(close, gt);
  if (q == std::string::npos || q > e) return false;
  std::string raw = s.substr(gt + 1, q - gt - 1);
  // strip CDATA wrappers and nested tags: text content only
  std::string txt;
  for (size_t i = 0; i < raw.size();) {
    if (raw.compare(i, 9, "<![CDATA[") == 0) {
      size_t z = raw.find("]]>", i);
      if (z == std::string::npos) z = raw.size();
      txt += raw.substr(i + 9, z - i - 9);
      i = z + 3;
    } else if (raw[i] == '<') {
      size_t z = raw.find('>', i);
      i = (z == std::string::npos) ? raw.size() : z + 1;
    } else {
      txt += raw[i++];
    }
  }
  *out = xml_decode(txt);
  return true;
}

bool is_true(const std::string& v) { return v == "true"; }

}  // namespace

int params_read_xml(const char* path, srs_params* p, std::string* err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    if (err) *err = std::string("cannot open parameter file ") + path;
    return SRS_ERR_IO;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  std::string s = ss.str();
  int* I = p->ints;
  double* R = p->reals;
  size_t pos = 0;
  int n_params = 0;
  while (true) {
    size_t b = s.find("<parameter", pos);
    if (b == std::string::npos) break;
    char c = s[b + 10];
    if (!(c == '>' || c == ' ' || c == '\t' || c == '\n' || c == '\r')) {
      pos = b + 10;
      continue;
    }
    size_t e = s.find("</parameter>", b);
    if (e == std::string::npos) break;
    pos = e + 12;
    ++n_params;
    std::string sym, val;
    if (!child_text(s, b, e, "symbol", &sym) || !child_text(s, b, e, "value", &val)) continue;
    const char* v = val.c_str();
    // Symbol table of cpu/InitFuncs.cpp:191-349.
    if (sym == "flag_noflux") I[I_FLAG_NO_FLUX_BOUNDARY] = is_true(val);
    else if (sym == "flag_nogating") I[I_FLAG_NO_GATING] = is_true(val);
    else if (sym == "flag_ffwd") I[I_GATING_FFWD] = is_true(val);
    else if (sym == "flag_use_clock") I[I_FLAG_CLOCK_SEED] = is_true(val);
    else if (sym == "flag_output_grid") I[I_OUTPUT_GRID_FLAG] = is_true(val);
    else if (sym == "protocol") {
      if (val == "gain") {
        I[I_FLAG_V_CLAMP] = 1;
        I[I_FLAG_FIDELITY_SIM] = 0;
      } else if (val == "fidelity") {
        I[I_FLAG_V_CLAMP] = 0;
        I[I_FLAG_FIDELITY_SIM] = 1;
      } else {
        I[I_FLAG_V_CLAMP] = 0;
        I[I_FLAG_FIDELITY_SIM] = 0;
      }
    } else if (sym == "flag_output_ryr_states") I[I_FLAG_RYR_OUT] = is_true(val);
    else if (sym == "sims_per_proc") I[I_N_SIMS] = std::atoi(v);
    else if (sym == "ryr_open_init") {
      if (!val.empty()) I[I_INIT_RYR] = std::atoi(v);
    } else if (sym == "c_min") R[R_C_MIN] = std::atof(v);
    else if (sym == "ryr_open_time") R[R_INIT_RYR_HOLD] = std::atof(v);
    else if (sym == "ryr_open_max") I[I_N_RYR_FIDELITY] = std::atoi(v);
    else if (sym == "v_clamp") R[R_V_CLAMP] = std::atof(v);
    else if (sym == "t_clamp") R[R_T_CLAMP] = std::atof(v);
    else if (sym == "t_final") R[R_T_FINAL] = std::atof(v);
    else if (sym == "t_step") R[R_T_STEP] = std::atof(v) * (1e-6);
    else if (sym == "states_interval") R[R_OUTPUT_STATES_INTERVAL] = std::atof(v);
    else if (sym == "grid_interval") R[R_OUTPUT_GRID_INTERVAL] = std::atof(v);
    else if (sym == "seed_base") I[I_RAND_SEED_0] = std::atoi(v);
    else if (sym == "seed_A") I[I_RAND_ADD_A] = std::atoi(v);
    else if (sym == "seed_B") I[I_RAND_ADD_B] = std::atoi(v);
    else if (sym == "CA_I") R[R_C_0_CA] = std::atof(v);
    else if (sym == "CA_SR") {
      R[R_C_0_CA_JSR] = std::atof(v);
      R[R_DEFAULT_CA_NSR] = std::atof(v);
    } else if (sym == "CA_O") R[R_CA_0] = std::atof(v);
    else if (sym == "V_M") R[R_DEFAULT_VM] = std::atof(v);
    else if (sym == "D_CA") R[R_D_CA] = std::atof(v);
    else if (sym == "D_CAJSR") R[R_D_CA_JSR] = std::atof(v);
    else if (sym == "D_ATP") R[R_D_ATP] = std::atof(v);
    else if (sym == "D_CMDN") R[R_D_CMDN] = std::atof(v);
    else if (sym == "D_DYE") R[R_D_DYE] = std::atof(v);
    else if (sym == "B_TOT_ATP") R[R_B_TOT_ATP] = std::atof(v);
    else if (sym == "K_OFF_ATP") R[R_K_OFF_ATP] = std::atof(v);
    else if (sym == "K_ON_ATP") R[R_K_ON_ATP] = std::atof(v);
    else if (sym == "B_TOT_CMDN") R[R_B_TOT_CMDN] = std::atof(v);
    else if (sym == "K_OFF_CMDN") R[R_K_OFF_CMDN] = std::atof(v);
    else if (sym == "K_ON_CMDN") R[R_K_ON_CMDN] = std::atof(v);
    else if (sym == "B_TOT_TRPN") R[R_B_TOT_TRPN] = std::atof(v);
    else if (sym == "K_OFF_TRPN") R[R_K_OFF_TRPN] = std::atof(v);
    else if (sym == "K_ON_TRPN") R[R_K_ON_TRPN] = std::atof(v);
    else if (sym == "B_TOT_SL") R[R_B_TOT_SL_HI] = std::atof(v);
    else if (sym == "K_D_SL") R[R_K_D_SL_HI] = std::atof(v);
    else if (sym == "B_TOT_DYE") R[R_B_TOT_DYE] = std::atof(v);
    else if (sym == "K_OFF_DYE") R[R_K_OFF_DYE] = std::atof(v);
    else if (sym == "K_ON_DYE") R[R_K_ON_DYE] = std::atof(v);
    else if (sym == "B_TOT_CSQN") R[R_B_T_JSR] = std::atof(v);
    else if (sym == "K_OFF_CSQN") R[R_K_OFF_CSQN] = std::atof(v);
    else if (sym == "K_ON_CSQN") R[R_K_ON_CSQN] = std::atof(v);
    else if (sym == "V_REFILL") R[R_V_REFILL] = std::atof(v);
    else if (sym == "V_RYR") R[R_V_RYR] = std::atof(v);
    else if (sym == "RYR_ETA") R[R_RYR_ETA] = std::atof(v);
    else if (sym == "RYR_A_STAR") R[R_RYR_A_STAR] = std::atof(v);
    else if (sym == "RYR_EPS_CC") R[R_RYR_EPS_CC] = std::atof(v);
    else if (sym == "RYR_EPS_OO") R[R_RYR_EPS_OO] = std::atof(v);
    else if (sym == "RYR_K_MINUS") R[R_RYR_K_MINUS] = std::atof(v);
    else if (sym == "RYR_K_PLUS") R[R_RYR_K_PLUS] = std::atof(v);
    else if (sym == "RYR_PHI_N") R[R_RYR_PHI_M] = std::atof(v);
    else if (sym == "RYR_PHI_KD") R[R_RYR_PHI_B] = std::atof(v);
    else if (sym == "K_D_I") R[R_K_D_i] = std::atof(v);
    else if (sym == "K_D_SR") R[R_K_D_SR] = std::atof(v);
    else if (sym == "A_P") R[R_A_P] = std::atof(v);
    else if (sym == "paramset_title") std::snprintf(p->chars[C_PARAM_TITLE], 255, "%s", v);
  }
  if (n_params == 0) {
    if (err) *err = "No parameters were found!";
    return SRS_ERR_IO;
  }
  return SRS_OK;
}

// ---------------------------------------------------------------------------
// Mesh files
// ---------------------------------------------------------------------------
namespace {

struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};

bool skip_line(FILE* f) {
  char line[4096];
  return std::fgets(line, sizeof(line), f) != nullptr;
}

}  // namespace

int mesh_read(const char* base, int flag_noflux, Mesh* m, std::string* err) {
  std::string b(base);
  auto fail = [&](int code, const std::string& msg) {
    if (err) *err = msg;
    return code;
  };
  // <base>_tet_properties.txt (cpu/InitFuncs.cpp:387-430)
  {
    std::string fn = b + "_tet_properties.txt";
    FileCloser fc{std::fopen(fn.c_str(), "r")};
    if (!fc.f) return fail(SRS_ERR_IO, "Error opening element properties file: " + fn);
    if (std::fscanf(fc.f, "%d\n", &m->N) != 1 || m->N <= 0)
      return fail(SRS_ERR_IO, "Error reading element property : number of elements");
    if (!skip_line(fc.f)) return fail(SRS_ERR_IO, "Error skipping header in " + fn);
    m->V0.resize(m->N);
    m->TT.resize(m->N);
    m->SR.resize(m->N);
    m->tropc.resize(m->N);
    m->domain.resize(m->N);
    for (int i = 0; i < m->N; ++i) {
      double j1, j2, j3;
      if (std::fscanf(fc.f, "%lg %lg %lg %lg %lg %lg %d %d\n", &j1, &j2, &j3, &m->V0[i], &m->TT[i],
                      &m->SR[i], &m->tropc[i], &m->domain[i]) != 8)
        return fail(SRS_ERR_IO, "Error reading element property data at line " + std::to_string(i + 3));
      if (!(m->V0[i] > 0.0)) return fail(SRS_ERR_MESH, "non-positive element volume");
      if (m->domain[i] != DOMAIN_CYTO && m->domain[i] != DOMAIN_JSR)
        return fail(SRS_ERR_MESH, "element domain must be 0 (cytosol) or 1 (JSR)");
    }
  }
  // <base>_face_properties.txt (cpu/InitFuncs.cpp:433-519)
  {
    std::string fn = b + "_face_properties.txt";
    FileCloser fc{std::fopen(fn.c_str(), "r")};
    if (!fc.f) return fail(SRS_ERR_IO, "Error opening face properties file: " + fn);
    if (std::fscanf(fc.f, "%d\n", &m->NF) != 1 || m->NF < 0)
      return fail(SRS_ERR_IO, "Error reading face property : number of faces.");
    if (!skip_line(fc.f)) return fail(SRS_ERR_IO, "Error skipping header in " + fn);
    m->ele1.resize(m->NF);
    m->ele2.resize(m->NF);
    m->ftype.resize(m->NF);
    m->faceC.resize(m->NF);
    for (int i = 0; i < m->NF; ++i) {
      double d[21];
      int t;
      int got = std::fscanf(fc.f,
                            "%d %d %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg "
                            "%lg %lg %lg %lg %lg %lg %d\n",
                            &m->ele1[i], &m->ele2[i], &d[0], &d[1], &d[2], &d[3], &d[4], &d[5],
                            &d[6], &d[7], &d[8], &d[9], &d[10], &d[11], &d[12], &d[13], &d[14],
                            &d[15], &d[16], &d[17], &d[18], &d[19], &d[20], &t);
      if (got != 24) return fail(SRS_ERR_IO, "Error reading face data at line " + std::to_string(i + 3));
      m->faceC[i] = d[20];
      switch (t) {  // (cpu/InitFuncs.cpp:494-514)
        case 0: t = FACE_DEFAULT; break;
        case 1: t = flag_noflux ? FACE_NOFLUX : FACE_BOUND; break;
        case 2: t = FACE_NOFLUX; break;
        case 3: t = FACE_NOFLUX; break;
        default: break;  // undefined input face type: kept, ignored by assembly
      }
      m->ftype[i] = t;
      if (m->ele1[i] < 0 || m->ele1[i] >= m->N || m->ele2[i] >= m->N)
        return fail(SRS_ERR_MESH, "face element index out of range at face " + std::to_string(i));
      if (t == FACE_DEFAULT && m->ele2[i] < 0)
        return fail(SRS_ERR_MESH, "interior face without a second element at face " + std::to_string(i));
    }
  }
  // <base>.node (cpu/InitFuncs.cpp:521-557)
  {
    std::string fn = b + ".node";
    FileCloser fc{std::fopen(fn.c_str(), "r")};
    if (!fc.f) return fail(SRS_ERR_IO, "Error opening node file: " + fn);
    if (std::fscanf(fc.f, "%d", &m->NN) != 1 || m->NN <= 0)
      return fail(SRS_ERR_IO, "Error node file - number of nodes");
    if (!skip_line(fc.f)) return fail(SRS_ERR_IO, "Error skipping header in " + fn);
    m->node_x.resize(m->NN);
    m->node_y.resize(m->NN);
    m->node_z.resize(m->NN);
    for (int i = 0; i < m->NN; ++i) {
      int j1;
      if (std::fscanf(fc.f, "%d %lg %lg %lg\n", &j1, &m->node_x[i], &m->node_y[i], &m->node_z[i]) != 4)
        return fail(SRS_ERR_IO, "Error reading node data at line " + std::to_string(i + 2));
    }
  }
  // <base>.ele (cpu/InitFuncs.cpp:559-595)
  {
    std::string fn = b + ".ele";
    FileCloser fc{std::fopen(fn.c_str(), "r")};
    if (!fc.f) return fail(SRS_ERR_IO, "Error opening element file: " + fn);
    if (!skip_line(fc.f)) return fail(SRS_ERR_IO, "Error skipping header in " + fn);
    m->ele_nodes.resize(4 * (size_t)m->N);
    for (int i = 0; i < m->N; ++i) {
      int j1, j2, *q = &m->ele_nodes[4 * (size_t)i];
      if (std::fscanf(fc.f, "%d %d %d %d %d %d\n", &j1, &q[0], &q[1], &q[2], &q[3], &j2) != 6)
        return fail(SRS_ERR_IO, "Error reading element data at line " + std::to_string(i + 2));
      for (int k = 0; k < 4; ++k) q[k]--;
    }
  }
  // <base>_lcc.txt (cpu/InitFuncs.cpp:597-624)
  {
    std::string fn = b + "_lcc.txt";
    FileCloser fc{std::fopen(fn.c_str(), "r")};
    if (!fc.f) return fail(SRS_ERR_IO, "Error opening file: " + fn);
    if (std::fscanf(fc.f, "%d\n", &m->NL) != 1 || m->NL < 0)
      return fail(SRS_ERR_IO, "Error reading number of LCCs");
    m->lcc_ele.resize(m->NL);
    for (int i = 0; i < m->NL; ++i)
      if (std::fscanf(fc.f, "%d\n", &m->lcc_ele[i]) != 1)
        return fail(SRS_ERR_IO, "Error reading LCC data at line " + std::to_string(i + 2));
  }
  // <base>_ryr.txt (cpu/InitFuncs.cpp:626-655)
  {
    std::string fn = b + "_ryr.txt";
    FileCloser fc{std::fopen(fn.c_str(), "r")};
    if (!fc.f) return fail(SRS_ERR_IO, "Error opening file: " + fn);
    if (std::fscanf(fc.f, "%d\n", &m->NR) != 1 || m->NR < 0)
      return fail(SRS_ERR_IO, "Error reading number of RyRs");
    m->ryr_ele.resize(m->NR);
    m->ryr_jsr.resize(m->NR);
    m->ryr_nb.resize(4 * (size_t)m->NR);
    for (int i = 0; i < m->NR; ++i)
      if (std::fscanf(fc.f, "%d %d %d %d %d %d\n", &m->ryr_ele[i], &m->ryr_jsr[i], &m->ryr_nb[4 * i],
                      &m->ryr_nb[4 * i + 1], &m->ryr_nb[4 * i + 2], &m->ryr_nb[4 * i + 3]) != 6)
        return fail(SRS_ERR_IO, "Error reading RyR data at line " + std::to_string(i + 2));
  }
  for (int i = 0; i < m->NR; ++i) {
    if (m->ryr_ele[i] < 0 || m->ryr_ele[i] >= m->N || m->ryr_jsr[i] < 0 || m->ryr_jsr[i] >= m->N)
      return fail(SRS_ERR_MESH, "RyR element index out of range");
    for (int k = 0; k < 4; ++k)
      if (m->ryr_nb[4 * i + k] >= m->NR) return fail(SRS_ERR_MESH, "RyR neighbour index out of range");
  }
  for (int i = 0; i < m->NL; ++i)
    if (m->lcc_ele[i] < 0 || m->lcc_ele[i] >= m->N) return fail(SRS_ERR_MESH, "LCC element index out of range");

  // Breadth-first renumbering from element 0 over faces with Ele_2 >= 0, each
  // element's neighbours taken in face order (cpu/InitFuncs.cpp:679-731).
  // Adjacency lists built in face order make this linear in N + NF; the
  // reference's quadratic membership scans give the same visiting order.
  const int N = m->N;
  std::vector<int> deg(N + 1, 0);
  for (int i = 0; i < m->NF; ++i)
    if (m->ele2[i] >= 0) {
      deg[m->ele1[i] + 1]++;
      deg[m->ele2[i] + 1]++;
    }
  for (int i = 0; i < N; ++i) deg[i + 1] += deg[i];
  std::vector<int> adj(deg[N]), fill(deg.begin(), deg.end() - 1);
  for (int i = 0; i < m->NF; ++i)
    if (m->ele2[i] >= 0) {
      adj[fill[m->ele1[i]]++] = m->ele2[i];
      adj[fill[m->ele2[i]]++] = m->ele1[i];
    }
  std::vector<int> visited;
  visited.reserve(N);
  std::vector<char> seen(N, 0);
  std::vector<int> queue;
  queue.reserve(N);
  queue.push_back(0);
  seen[0] = 1;
  for (size_t h = 0; h < queue.size(); ++h) {
    int v = queue[h];
    visited.push_back(v);
    for (int k = deg[v]; k < deg[v + 1]; ++k) {
      int u = adj[k];
      if (!seen[u]) {
        seen[u] = 1;
        queue.push_back(u);
      }
    }
  }
  if ((int)visited.size() != N)
    return fail(SRS_ERR_MESH, "mesh is not connected through its faces (renumbering reaches " +
                                  std::to_string(visited.size()) + " of " + std::to_string(N) +
                                  " elements)");
  std::vector<int> old2new(N);
  for (int i = 0; i < N; ++i) old2new[visited[i]] = i;
  auto permute_d = [&](std::vector<double>& a) {
    std::vector<double> t(N);
    for (int i = 0; i < N; ++i) t[i] = a[visited[i]];
    a.swap(t);
  };
  auto permute_i = [&](std::vector<int>& a) {
    std::vector<int> t(N);
    for (int i = 0; i < N; ++i) t[i] = a[visited[i]];
    a.swap(t);
  };
  permute_d(m->V0);
  permute_d(m->TT);
  permute_d(m->SR);
  permute_i(m->tropc);
  permute_i(m->domain);
  {
    std::vector<int> t(4 * (size_t)N);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < 4; ++k) t[4 * (size_t)i + k] = m->ele_nodes[4 * (size_t)visited[i] + k];
    m->ele_nodes.swap(t);
  }
  for (int i = 0; i < m->NF; ++i) {
    m->ele1[i] = old2new[m->ele1[i]];
    if (m->ele2[i] >= 0) m->ele2[i] = old2new[m->ele2[i]];
  }
  for (int i = 0; i < m->NR; ++i) {
    m->ryr_ele[i] = old2new[m->ryr_ele[i]];
    m->ryr_jsr[i] = old2new[m->ryr_jsr[i]];
  }
  for (int i = 0; i < m->NL; ++i) m->lcc_ele[i] = old2new[m->lcc_ele[i]];
  m->order = visited;
  return SRS_OK;
}

RestValues rest_values(const srs_params& p) {
  // cpu/InitFuncs.cpp:895-917
  const double* R = p.reals;
  RestValues r;
  r.ca0 = R[R_C_0_CA];
  r.ca0_jsr = R[R_C_0_CA_JSR];
  double Kd;
  Kd = R[R_K_OFF_TRPN] / R[R_K_ON_TRPN];
  r.trpn = r.ca0 * R[R_B_TOT_TRPN] / (Kd + r.ca0);
  Kd = R[R_K_OFF_CSQN] / R[R_K_ON_CSQN];
  r.csqn = r.ca0_jsr * R[R_B_T_JSR] / (Kd + r.ca0_jsr);
  Kd = R[R_K_OFF_ATP] / R[R_K_ON_ATP];
  r.atp = r.ca0 * R[R_B_TOT_ATP] / (Kd + r.ca0);
  Kd = R[R_K_OFF_CMDN] / R[R_K_ON_CMDN];
  r.cmdn = r.ca0 * R[R_B_TOT_CMDN] / (Kd + r.ca0);
  Kd = R[R_K_OFF_DYE] / R[R_K_ON_DYE];
  r.dye = r.ca0 * R[R_B_TOT_DYE] / (Kd + r.ca0);
  return r;
}

void initial_states(const Mesh& m, const srs_params& p, std::vector<double>* states) {
  // cpu/InitFuncs.cpp:928-954
  RestValues rv = rest_values(p);
  const int N = m.N;
  states->assign((size_t)N_SPECIES * N, 0.0);
  double* S = states->data();
  for (int j = 0; j < N; ++j) {
    if (m.domain[j] == DOMAIN_CYTO) {
      S[SP_CA * N + j] = rv.ca0;
      S[SP_TRPN * N + j] = rv.trpn * m.tropc[j];
      S[SP_ATP * N + j] = rv.atp;
      S[SP_CMDN * N + j] = rv.cmdn;
      S[SP_DYE * N + j] = rv.dye;
      S[SP_CSQN * N + j] = 0.0;  // left unset by the reference; never read
    } else {
      S[SP_CA * N + j] = rv.ca0_jsr;
      S[SP_TRPN * N + j] = 0;
      S[SP_CSQN * N + j] = rv.csqn;
      S[SP_ATP * N + j] = 0;
      S[SP_CMDN * N + j] = 0;
      S[SP_DYE * N + j] = 0;
    }
  }
}

int assemble_operator(const Mesh& m, const srs_params& p, Operator* op, std::string* err) {
  const int N = m.N;
  // Row-wise accumulation in face order reproduces the std::map<(i,j),double>
  // accumulation of cpu/InitFuncs.cpp:1073-1112 term by term (each (i,j) key
  // receives its contributions in face order; keys are visited row-major).
  std::vector<double> diag(N, 0.0);
  std::vector<std::vector<std::pair<int, double>>> off(N);
  for (int f = 0; f < m.NF; ++f) {
    int t1 = m.ele1[f], t2 = m.ele2[f];
    double k1 = m.faceC[f] / m.V0[t1];  // diff = 1 (cpu/InitFuncs.cpp:1081-1083)
    if (m.ftype[f] == FACE_DEFAULT) {
      off[t1].push_back({t2, k1});
      diag[t1] += -k1;
      double k2 = m.faceC[f] / m.V0[t2];
      off[t2].push_back({t1, k2});
      diag[t2] += -k2;
    } else if (m.ftype[f] == FACE_BOUND) {
      diag[t1] += -k1;
    }
  }
  op->aij.assign(5 * (size_t)N, 0.0);
  op->nij.resize(4 * (size_t)N);
  op->max_diag = 0.0;
  for (int i = 0; i < N; ++i) {
    for (int k = 0; k < 4; ++k) op->nij[4 * (size_t)i + k] = i;
    auto& row = off[i];
    // combine duplicate columns in face order, then order by column
    std::stable_sort(row.begin(), row.end(),
                     [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
                       return a.first < b.first;
                     });
    std::vector<std::pair<int, double>> merged;
    for (auto& e : row) {
      if (!merged.empty() && merged.back().first == e.first) merged.back().second += e.second;
      else merged.push_back(e);
    }
    // Ordered entries of the row: the diagonal sits at column i.
    int nf = 0;
    if (diag[i] != 0) op->aij[5 * (size_t)i] = diag[i];
    for (auto& e : merged) {
      if (e.second == 0) continue;  // zero entries are not stored (:1276-1293)
      if (nf >= 4) {
        if (err) *err = "element " + std::to_string(i) + " has more than 4 neighbours";
        return SRS_ERR_MESH;
      }
      op->aij[5 * (size_t)i + 1 + nf] = e.second;
      op->nij[4 * (size_t)i + nf] = e.first;
      ++nf;
    }
    op->max_diag = std::max(op->max_diag, std::fabs(diag[i]));
  }
  // Boundary rates (cpu/InitFuncs.cpp:1013-1026) with boundary values from
  // ResetDefaultGridStates (cpu/InitFuncs.cpp:920-925).
  RestValues rv = rest_values(p);
  op->boundary_value[SP_CA] = rv.ca0;
  op->boundary_value[SP_TRPN] = rv.trpn;
  op->boundary_value[SP_CSQN] = 0;
  op->boundary_value[SP_ATP] = rv.atp;
  op->boundary_value[SP_CMDN] = rv.cmdn;
  op->boundary_value[SP_DYE] = rv.dye;
  double D[N_SPECIES];
  diffusion_by_species(p, D);
  op->br.assign((size_t)N_SPECIES * N, 0.0);
  op->kb.assign(N, 0.0);
  for (int k = 0; k < N_SPECIES; ++k)
    for (int f = 0; f < m.NF; ++f) {
      if (m.ftype[f] != FACE_BOUND) continue;
      int t1 = m.ele1[f];
      op->br[(size_t)k * N + t1] += D[k] * (m.faceC[f]) * op->boundary_value[k] / m.V0[t1];
    }
  for (int f = 0; f < m.NF; ++f)
    if (m.ftype[f] == FACE_BOUND) op->kb[m.ele1[f]] += m.faceC[f] / m.V0[m.ele1[f]];
  return SRS_OK;
}

std::vector<int> rcm_order_by_domain(const Mesh& m, const Operator& op) {
  // Reverse Cuthill-McKee on the operator graph, one domain at a time
  // (cytosol first, then JSR), each component started from a
  // minimum-degree element.
  const int N = m.N;
  std::vector<int> degree(N, 0);
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < 4; ++k)
      if (op.nij[4 * (size_t)i + k] != i && op.aij[5 * (size_t)i + 1 + k] != 0) degree[i]++;
  std::vector<int> perm;
  perm.reserve(N);
  std::vector<char> seen(N, 0);
  for (int dom = 0; dom <= 1; ++dom) {
    std::vector<int> cand;
    for (int i = 0; i < N; ++i)
      if (m.domain[i] == dom) cand.push_back(i);
    std::stable_sort(cand.begin(), cand.end(),
                     [&](int a, int b) { return degree[a] < degree[b]; });
    std::vector<int> dom_order;
    for (int start : cand) {
      if (seen[start]) continue;
      std::vector<int> comp;
      comp.push_back(start);
      seen[start] = 1;
      for (size_t h = 0; h < comp.size(); ++h) {
        int v = comp[h];
        int nb[4], nn = 0;
        for (int k = 0; k < 4; ++k) {
          int u = op.nij[4 * (size_t)v + k];
          if (u != v && op.aij[5 * (size_t)v + 1 + k] != 0 && !seen[u] && m.domain[u] == dom)
            nb[nn++] = u;
        }
        std::sort(nb, nb + nn, [&](int a, int b) {
          return degree[a] != degree[b] ? degree[a] < degree[b] : a < b;
        });
        for (int q = 0; q < nn; ++q) {
          seen[nb[q]] = 1;
          comp.push_back(nb[q]);
        }
      }
      dom_order.insert(dom_order.end(), comp.begin(), comp.end());
    }
    std::reverse(dom_order.begin(), dom_order.end());
    perm.insert(perm.end(), dom_order.begin(), dom_order.end());
  }
  return perm;
}

Schedule make_schedule(const srs_params& p, double t0) {
  // Replays t += dt of cpu/RunSimulation.cpp:522-574 (including the
  // floor(t/I) > floor((t - dt_last)/I) output test at :552).
  Schedule s;
  const double dt = p.reals[R_T_STEP];
  const double T_FINAL = p.reals[R_T_FINAL];
  const double I_states = p.reals[R_OUTPUT_STATES_INTERVAL];
  const double I_grid = p.reals[R_OUTPUT_GRID_INTERVAL];
  const bool grid = p.ints[I_OUTPUT_GRID_FLAG] != 0;
  double t = t0, dt_last = 0;
  int64_t n = 0;
  bool clamp = p.ints[I_FLAG_V_CLAMP] != 0;
  bool hold = p.ints[I_INIT_RYR] != -1;
  while (t <= T_FINAL) {
    if (clamp && s.clamp_end_step < 0 && !(t <= p.reals[R_T_CLAMP])) s.clamp_end_step = n;
    if (hold && s.hold_end_step < 0 && !(t < p.reals[R_INIT_RYR_HOLD])) s.hold_end_step = n;
    // grid files are tested first, states rows second (cpu/RunSimulation.cpp:545-553)
    if (grid && std::floor(t / I_grid) > std::floor((t - dt_last) / I_grid)) {
      s.grid_steps.push_back(n);
      s.grid_times.push_back(t);
    }
    if (std::floor(t / I_states) > std::floor((t - dt_last) / I_states)) {
      s.tick_steps.push_back(n);
      s.tick_times.push_back(t);
    }
    t += dt;
    dt_last = dt;
    ++n;
  }
  if (clamp && s.clamp_end_step < 0) s.clamp_end_step = n;
  if (hold && s.hold_end_step < 0) s.hold_end_step = n;
  s.n_steps = n;
  s.t_end = t;
  return s;
}

int64_t first_step_at_or_after(const srs_params& p, double T) {
  const double dt = p.reals[R_T_STEP];
  const double T_FINAL = p.reals[R_T_FINAL];
  double t = 0;
  int64_t n = 0;
  while (t <= T_FINAL) {
    if (t >= T) return n;
    t += dt;
    ++n;
  }
  return n;
}

int states_row(const Mesh& m, const srs_params& p, const double* ca, const int* ryr_state,
               const int* lcc_state, const int* lccv_state, double V, double t, float* row,
               int row_cap) {
  // WriteToStateFiles (cpu/OutputFuncs.cpp:241-350)
  const double* R = p.reals;
  int k = 0;
  row[k++] = (float)t;
  double i_ryr = 0;
  for (int i = 0; i < m.NR; ++i) {
    double CaJSR = ca[m.ryr_jsr[i]];
    double CaSS = ca[m.ryr_ele[i]];
    i_ryr += ryr_state[i] * R[R_V_RYR] * (CaJSR - CaSS) * (R[R_V_CELL]) * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_ryr;
  int n_open = 0;
  for (int i = 0; i < m.NR; ++i) n_open += ryr_state[i];
  row[k++] = (float)n_open;
  int n_lcc = 0;
  for (int i = 0; i < m.NL; ++i)
    if (lccv_state[i] == 2 && (lcc_state[i] == 6 || lcc_state[i] == 12)) n_lcc++;
  row[k++] = (float)n_lcc;
  const double P_CaL = (9.13e-13) * (1e12) * (1e-3);
  const double F = 96.5;
  const double RT = 310 * 8.314;
  const double F_over_RT = F / RT;
  if (std::fabs(V) < 1e-6) V = 1e-6;
  double i_lcc = 0;
  for (int i = 0; i < m.NL; ++i) {
    double CA_DYAD = ca[m.lcc_ele[i]];
    if ((lcc_state[i] == 6 || lcc_state[i] == 12) && lccv_state[i] == 2)
      i_lcc += -P_CaL * V * (2 * F_over_RT) * (CA_DYAD * std::exp(2 * V * F_over_RT) - 0.34 * R[R_CA_0]) /
               (std::exp(2 * V * F_over_RT) - 1) * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_lcc;
  double mean_sr = 0;
  for (int i = 0; i < m.NR; ++i) mean_sr += ca[m.ryr_jsr[i]];
  mean_sr /= m.NR;
  row[k++] = (float)mean_sr;
  double mean_i = 0;
  for (int i = 0; i < m.NR; ++i) mean_i += ca[m.ryr_ele[i]];
  mean_i /= m.NR;
  row[k++] = (float)mean_i;
  if (p.ints[I_FLAG_RYR_OUT]) {
    for (int i = 0; i < m.NR && k < row_cap; ++i) row[k++] = (float)ryr_state[i];
  }
  return k;
}

int write_grid_vtk(const char* path, const Mesh& m, int run, int rank, int n, double t,
                   const double* ca, const double* dye, const int* ryr_state) {
  // WriteToGridFiles (cpu/OutputFuncs.cpp:69-182), same text layout.
  FILE* f = std::fopen(path, "w");
  if (!f) return SRS_ERR_IO;
  std::fprintf(f, "# vtk DataFile Version 3.0\n");
  std::fprintf(f, "Grid data for run %d-%d-%d at t = %f\n", run, rank, n, t);
  std::fprintf(f, "ASCII\n\n");
  std::fprintf(f, "DATASET UNSTRUCTURED_GRID\n");
  std::fprintf(f, "POINTS %d float\n", m.NN);
  for (int j = 0; j < m.NN; ++j) std::fprintf(f, "%f %f %f\n", m.node_x[j], m.node_y[j], m.node_z[j]);
  std::fprintf(f, "\nCELLS %d %d\n", m.N, 5 * m.N);
  for (int j = 0; j < m.N; ++j)
    std::fprintf(f, "4 %d %d %d %d\n", m.ele_nodes[4 * (size_t)j], m.ele_nodes[4 * (size_t)j + 1],
                 m.ele_nodes[4 * (size_t)j + 2], m.ele_nodes[4 * (size_t)j + 3]);
  std::fprintf(f, "\nCELL_TYPES %d\n", m.N);
  for (int j = 0; j < m.N; ++j) std::fprintf(f, "10\n");
  std::fprintf(f, "\nCELL_DATA %d\n", m.N);
  std::fprintf(f, "SCALARS C_CA float\n");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  for (int j = 0; j < m.N; ++j) std::fprintf(f, "%f\n", ca[j]);
  std::fprintf(f, "SCALARS C_DYE float\n");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  for (int j = 0; j < m.N; ++j) std::fprintf(f, "%f\n", dye[j]);
  std::fprintf(f, "SCALARS B_RYR int\n");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  std::vector<int> b(m.N, 0);
  for (int i = 0; i < m.NR; ++i) {
    b[m.ryr_ele[i]] = 1;
    if (ryr_state[i]) b[m.ryr_ele[i]] = 2;
  }
  for (int j = 0; j < m.N; ++j) std::fprintf(f, "%d\n", b[j]);
  std::fprintf(f, "SCALARS B_JSR int\n");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  for (int j = 0; j < m.N; ++j) std::fprintf(f, "%d\n", m.domain[j] == DOMAIN_JSR ? 1 : 0);
  std::fprintf(f, "SCALARS B_LCC int\n");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  std::fill(b.begin(), b.end(), 0);
  for (int i = 0; i < m.NL; ++i) b[m.lcc_ele[i]] = 1;
  for (int j = 0; j < m.N; ++j) std::fprintf(f, "%d\n", b[j]);
  std::fclose(f);
  return SRS_OK;
}

}  // namespace srs
