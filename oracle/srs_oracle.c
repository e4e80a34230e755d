/*
 * srs_oracle.c — CPU oracle of the spark timestep.  TEST INFRASTRUCTURE:
 * only tests/, the smoke check and bench.py's CPU-baseline leg use it, to
 * compare against; the product never does.
 *
 * Each function restates the reference function it names
 * (mwalker174/srs, cpu/*.cpp) in plain C99, keeping its arithmetic order,
 * so that with the same inputs the FP64 results agree bit for bit with the
 * reference's own cpu/RunSimulation.cpp (compiled in oracle/_ref).
 * Compile with -ffp-contract=off.
 */
#include "srs_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---- parameter indices (cpu/parameters.h:18-92) ------------------------ */
enum {
  OI_FLAG_CLOCK_SEED = 2, OI_RAND_SEED_0 = 3, OI_RAND_ADD_A = 4, OI_RAND_ADD_B = 5,
  OI_N_RYR_FIDELITY = 10, OI_FLAG_LCC = 11, OI_LCC_INDEX = 12, OI_FLAG_V_CLAMP = 13,
  OI_FLAG_NO_GATING = 14, OI_FLAG_RYR_OUT = 16, OI_INIT_RYR = 18, OI_FLAG_FIDELITY_SIM = 1
};
enum {
  OR_T_FINAL = 0, OR_T_STEP = 1, OR_STATES_INTERVAL = 2, OR_C_MIN = 4, OR_D_CA = 5, OR_D_ATP = 7,
  OR_D_CMDN = 8, OR_D_TRPN = 9, OR_D_CSQN = 10, OR_D_DYE = 11, OR_C_0_CA = 13, OR_C_0_CA_JSR = 14,
  OR_DEFAULT_VM = 15, OR_DEFAULT_CA_NSR = 16, OR_CA_0 = 17, OR_B_TOT_ATP = 18, OR_K_OFF_ATP = 19,
  OR_K_ON_ATP = 20, OR_B_TOT_CMDN = 21, OR_K_OFF_CMDN = 22, OR_K_ON_CMDN = 23, OR_B_TOT_TRPN = 24,
  OR_K_OFF_TRPN = 25, OR_K_ON_TRPN = 26, OR_B_TOT_SL_HI = 27, OR_K_D_SL_HI = 28,
  OR_B_TOT_SL_LO = 29, OR_K_D_SL_LO = 30, OR_B_TOT_DYE = 31, OR_K_OFF_DYE = 32, OR_K_ON_DYE = 33,
  OR_B_T_JSR = 34, OR_V_REFILL = 36, OR_V_RYR = 37, OR_V_CELL = 38, OR_K_ON_CSQN = 39,
  OR_K_OFF_CSQN = 40, OR_RYR_ETA = 41, OR_RYR_A_STAR = 42, OR_RYR_EPS_CC = 43,
  OR_RYR_EPS_OO = 44, OR_RYR_K_PLUS = 45, OR_RYR_K_MINUS = 46, OR_RYR_PHI_M = 47,
  OR_RYR_PHI_B = 48, OR_K_D_i = 49, OR_K_D_SR = 50, OR_A_P = 51, OR_LCC_DURATION = 52,
  OR_T_CLAMP = 53, OR_V_CLAMP = 54, OR_INIT_RYR_HOLD = 55
};
enum { S_CA = 0, S_ATP = 1, S_CMDN = 2, S_TRPN = 3, S_CSQN = 4, S_DYE = 5 };

struct or_mesh {
  int N, NF, NN, NR, NL;
  double *V0, *TT, *SR;
  int *tropc, *domain;
  int *ele1, *ele2, *ftype;
  double* faceC;
  int *ryr_ele, *ryr_jsr, *ryr_nb, *lcc_ele;
  int* order;
  double* aij;
  int* nij;
  double* br;
  double* scratch; /* States_Buffer of cpu/parameters.h:165 (6N) */
};

static void skipline(FILE* f) {
  char line[4096];
  if (!fgets(line, sizeof(line), f)) return;
}

/* ReadGrid (cpu/InitFuncs.cpp:384-813). */
int or_mesh_load(const char* base, int flag_noflux, const double* reals, or_mesh** out) {
  char fn[1024];
  FILE* f;
  int i, j;
  or_mesh* m = (or_mesh*)calloc(1, sizeof(or_mesh));
  snprintf(fn, sizeof(fn), "%s_tet_properties.txt", base);
  f = fopen(fn, "r");
  if (!f) return -2;
  if (fscanf(f, "%d\n", &m->N) != 1) return -2;
  skipline(f);
  m->V0 = malloc(sizeof(double) * m->N);
  m->TT = malloc(sizeof(double) * m->N);
  m->SR = malloc(sizeof(double) * m->N);
  m->tropc = malloc(sizeof(int) * m->N);
  m->domain = malloc(sizeof(int) * m->N);
  for (i = 0; i < m->N; ++i) {
    double a, b, c;
    if (fscanf(f, "%lg %lg %lg %lg %lg %lg %d %d\n", &a, &b, &c, &m->V0[i], &m->TT[i], &m->SR[i],
               &m->tropc[i], &m->domain[i]) != 8)
      return -2;
  }
  fclose(f);
  snprintf(fn, sizeof(fn), "%s_face_properties.txt", base);
  f = fopen(fn, "r");
  if (!f) return -2;
  if (fscanf(f, "%d\n", &m->NF) != 1) return -2;
  skipline(f);
  m->ele1 = malloc(sizeof(int) * m->NF);
  m->ele2 = malloc(sizeof(int) * m->NF);
  m->ftype = malloc(sizeof(int) * m->NF);
  m->faceC = malloc(sizeof(double) * m->NF);
  for (i = 0; i < m->NF; ++i) {
    double d[21];
    int t;
    if (fscanf(f,
               "%d %d %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg "
               "%lg %lg %lg %d\n",
               &m->ele1[i], &m->ele2[i], &d[0], &d[1], &d[2], &d[3], &d[4], &d[5], &d[6], &d[7],
               &d[8], &d[9], &d[10], &d[11], &d[12], &d[13], &d[14], &d[15], &d[16], &d[17], &d[18],
               &d[19], &d[20], &t) != 24)
      return -2;
    m->faceC[i] = d[20];
    /* FACE_DEFAULT 0, FACE_BOUND 1, FACE_NOFLUX 2 (cpu/InitFuncs.cpp:494-514) */
    if (t == 0) t = 0;
    else if (t == 1) t = flag_noflux ? 2 : 1;
    else if (t == 2 || t == 3) t = 2;
    m->ftype[i] = t;
  }
  fclose(f);
  snprintf(fn, sizeof(fn), "%s.node", base);
  f = fopen(fn, "r");
  if (!f) return -2;
  if (fscanf(f, "%d", &m->NN) != 1) return -2;
  fclose(f);
  snprintf(fn, sizeof(fn), "%s_lcc.txt", base);
  f = fopen(fn, "r");
  if (!f) return -2;
  if (fscanf(f, "%d\n", &m->NL) != 1) return -2;
  m->lcc_ele = malloc(sizeof(int) * (m->NL + 1));
  for (i = 0; i < m->NL; ++i)
    if (fscanf(f, "%d\n", &m->lcc_ele[i]) != 1) return -2;
  fclose(f);
  snprintf(fn, sizeof(fn), "%s_ryr.txt", base);
  f = fopen(fn, "r");
  if (!f) return -2;
  if (fscanf(f, "%d\n", &m->NR) != 1) return -2;
  m->ryr_ele = malloc(sizeof(int) * (m->NR + 1));
  m->ryr_jsr = malloc(sizeof(int) * (m->NR + 1));
  m->ryr_nb = malloc(sizeof(int) * 4 * (m->NR + 1));
  for (i = 0; i < m->NR; ++i)
    if (fscanf(f, "%d %d %d %d %d %d\n", &m->ryr_ele[i], &m->ryr_jsr[i], &m->ryr_nb[4 * i],
               &m->ryr_nb[4 * i + 1], &m->ryr_nb[4 * i + 2], &m->ryr_nb[4 * i + 3]) != 6)
      return -2;
  fclose(f);

  /* Breadth-first renumbering exactly as written (cpu/InitFuncs.cpp:679-731):
   * a FIFO of vertices, neighbours found by scanning the face list, skipped
   * when already queued or visited.  Quadratic; meant for small meshes. */
  {
    int nf2 = 0, *e1 = malloc(sizeof(int) * m->NF), *e2 = malloc(sizeof(int) * m->NF);
    int *queue = malloc(sizeof(int) * (m->N + 1)), qh = 0, qt = 0;
    int* visited = malloc(sizeof(int) * m->N);
    int nvis = 0;
    char* inq = calloc(m->N, 1);
    char* isvis = calloc(m->N, 1);
    for (i = 0; i < m->NF; ++i)
      if (m->ele2[i] >= 0) {
        e1[nf2] = m->ele1[i];
        e2[nf2] = m->ele2[i];
        ++nf2;
      }
    queue[qt++] = 0;
    inq[0] = 1;
    while (qh < qt) {
      int v = queue[qh++];
      inq[v] = 0;
      visited[nvis++] = v;
      isvis[v] = 1;
      for (i = 0; i < nf2; ++i) {
        if (e1[i] == v || e2[i] == v) {
          int nb = (e1[i] == v) ? e2[i] : e1[i];
          if (!inq[nb] && !isvis[nb]) {
            queue[qt++] = nb;
            inq[nb] = 1;
          }
        }
      }
    }
    if (nvis != m->N) return -3;
    {
      int* o2n = malloc(sizeof(int) * m->N);
      double *V0 = malloc(sizeof(double) * m->N), *TT = malloc(sizeof(double) * m->N),
             *SR = malloc(sizeof(double) * m->N);
      int *tr = malloc(sizeof(int) * m->N), *dm = malloc(sizeof(int) * m->N);
      for (i = 0; i < m->N; ++i) o2n[visited[i]] = i;
      for (i = 0; i < m->N; ++i) {
        V0[i] = m->V0[visited[i]];
        TT[i] = m->TT[visited[i]];
        SR[i] = m->SR[visited[i]];
        tr[i] = m->tropc[visited[i]];
        dm[i] = m->domain[visited[i]];
      }
      free(m->V0);
      free(m->TT);
      free(m->SR);
      free(m->tropc);
      free(m->domain);
      m->V0 = V0;
      m->TT = TT;
      m->SR = SR;
      m->tropc = tr;
      m->domain = dm;
      for (j = 0; j < m->NF; ++j) {
        m->ele1[j] = o2n[m->ele1[j]];
        if (m->ele2[j] >= 0) m->ele2[j] = o2n[m->ele2[j]];
      }
      for (j = 0; j < m->NR; ++j) {
        m->ryr_ele[j] = o2n[m->ryr_ele[j]];
        m->ryr_jsr[j] = o2n[m->ryr_jsr[j]];
      }
      for (j = 0; j < m->NL; ++j) m->lcc_ele[j] = o2n[m->lcc_ele[j]];
      free(o2n);
    }
    m->order = visited;
    free(e1);
    free(e2);
    free(queue);
    free(inq);
    free(isvis);
  }

  /* InitializeExplicitSparseMatrixFast (cpu/InitFuncs.cpp:1058-1322): a map
   * keyed by (row, col) accumulating in face order, read out row-major. */
  {
    int N = m->N, f2;
    int* cnt = calloc(N, sizeof(int));
    int* col = malloc(sizeof(int) * N * 8);
    double* val = malloc(sizeof(double) * N * 8);
    double* diag = calloc(N, sizeof(double));
    char* hasdiag = calloc(N, 1);
    for (f2 = 0; f2 < m->NF; ++f2) {
      int t1 = m->ele1[f2], t2 = m->ele2[f2];
      double diff = 1;
      double k1 = diff * (m->faceC[f2]) / m->V0[t1];
      if (m->ftype[f2] == 0) {
        int q, found = -1;
        for (q = 0; q < cnt[t1]; ++q)
          if (col[t1 * 8 + q] == t2) found = q;
        if (found < 0) {
          col[t1 * 8 + cnt[t1]] = t2;
          val[t1 * 8 + cnt[t1]] = 0.0;
          found = cnt[t1]++;
        }
        val[t1 * 8 + found] += k1;
        diag[t1] += -k1;
        hasdiag[t1] = 1;
        {
          double k2 = diff * (m->faceC[f2]) / m->V0[t2];
          found = -1;
          for (q = 0; q < cnt[t2]; ++q)
            if (col[t2 * 8 + q] == t1) found = q;
          if (found < 0) {
            col[t2 * 8 + cnt[t2]] = t1;
            val[t2 * 8 + cnt[t2]] = 0.0;
            found = cnt[t2]++;
          }
          val[t2 * 8 + found] += k2;
          diag[t2] += -k2;
          hasdiag[t2] = 1;
        }
      } else if (m->ftype[f2] == 1) {
        diag[t1] += -k1;
        hasdiag[t1] = 1;
      }
    }
    m->aij = calloc(5 * (size_t)N, sizeof(double));
    m->nij = malloc(sizeof(int) * 4 * (size_t)N);
    for (i = 0; i < N; ++i) {
      int q, r, nfc = 0;
      for (q = 0; q < 4; ++q) m->nij[4 * i + q] = i;
      /* sort this row's off-diagonal entries by column (insertion sort) */
      for (q = 1; q < cnt[i]; ++q) {
        int c = col[i * 8 + q];
        double v = val[i * 8 + q];
        r = q - 1;
        while (r >= 0 && col[i * 8 + r] > c) {
          col[i * 8 + r + 1] = col[i * 8 + r];
          val[i * 8 + r + 1] = val[i * 8 + r];
          --r;
        }
        col[i * 8 + r + 1] = c;
        val[i * 8 + r + 1] = v;
      }
      if (hasdiag[i] && diag[i] != 0) m->aij[5 * i] = diag[i];
      for (q = 0; q < cnt[i]; ++q) {
        if (val[i * 8 + q] == 0) continue;
        if (nfc >= 4) return -3;
        m->aij[5 * i + 1 + nfc] = val[i * 8 + q];
        m->nij[4 * i + nfc] = col[i * 8 + q];
        ++nfc;
      }
    }
    free(cnt);
    free(col);
    free(val);
    free(diag);
    free(hasdiag);
  }
  /* Boundary rates (cpu/InitFuncs.cpp:1013-1026) with the boundary values of
   * ResetDefaultGridStates (cpu/InitFuncs.cpp:895-925). */
  {
    int N = m->N, k, f2;
    double ca0 = reals[OR_C_0_CA], Kd, Bv[6], Df[6];
    Kd = reals[OR_K_OFF_TRPN] / reals[OR_K_ON_TRPN];
    Bv[S_TRPN] = ca0 * reals[OR_B_TOT_TRPN] / (Kd + ca0);
    Kd = reals[OR_K_OFF_ATP] / reals[OR_K_ON_ATP];
    Bv[S_ATP] = ca0 * reals[OR_B_TOT_ATP] / (Kd + ca0);
    Kd = reals[OR_K_OFF_CMDN] / reals[OR_K_ON_CMDN];
    Bv[S_CMDN] = ca0 * reals[OR_B_TOT_CMDN] / (Kd + ca0);
    Kd = reals[OR_K_OFF_DYE] / reals[OR_K_ON_DYE];
    Bv[S_DYE] = ca0 * reals[OR_B_TOT_DYE] / (Kd + ca0);
    Bv[S_CA] = ca0;
    Bv[S_CSQN] = 0;
    Df[0] = reals[OR_D_CA];
    Df[1] = reals[OR_D_ATP];
    Df[2] = reals[OR_D_CMDN];
    Df[3] = reals[OR_D_TRPN];
    Df[4] = reals[OR_D_CSQN];
    Df[5] = reals[OR_D_DYE];
    m->br = calloc(6 * (size_t)N, sizeof(double));
    for (k = 0; k < 6; ++k)
      for (f2 = 0; f2 < m->NF; ++f2)
        if (m->ftype[f2] == 1) {
          int t1 = m->ele1[f2];
          m->br[k * N + t1] += Df[k] * (m->faceC[f2]) * Bv[k] / m->V0[t1];
        }
  }
  *out = m;
  return 0;
}

void or_mesh_free(or_mesh* m) {
  if (!m) return;
  free(m->V0);
  free(m->TT);
  free(m->SR);
  free(m->tropc);
  free(m->domain);
  free(m->ele1);
  free(m->ele2);
  free(m->ftype);
  free(m->faceC);
  free(m->ryr_ele);
  free(m->ryr_jsr);
  free(m->ryr_nb);
  free(m->lcc_ele);
  free(m->order);
  free(m->aij);
  free(m->nij);
  free(m->br);
  free(m->scratch);
  free(m);
}

void or_mesh_counts(const or_mesh* m, int* c) {
  int i, nj = 0;
  for (i = 0; i < m->N; ++i) nj += m->domain[i] == 1;
  c[0] = m->N;
  c[1] = m->NF;
  c[2] = m->NN;
  c[3] = m->NR;
  c[4] = m->NL;
  c[5] = nj;
}
void or_mesh_operator(const or_mesh* m, double* aij, int* nij, double* br) {
  memcpy(aij, m->aij, sizeof(double) * 5 * m->N);
  memcpy(nij, m->nij, sizeof(int) * 4 * m->N);
  memcpy(br, m->br, sizeof(double) * 6 * m->N);
}
void or_mesh_elements(const or_mesh* m, double* v0, double* tt, int* domain, int* tropc, int* order) {
  memcpy(v0, m->V0, sizeof(double) * m->N);
  memcpy(tt, m->TT, sizeof(double) * m->N);
  memcpy(domain, m->domain, sizeof(int) * m->N);
  memcpy(tropc, m->tropc, sizeof(int) * m->N);
  memcpy(order, m->order, sizeof(int) * m->N);
}
void or_mesh_channels(const or_mesh* m, int* ryr_ele, int* ryr_jsr, int* ryr_nb, int* lcc_ele) {
  memcpy(ryr_ele, m->ryr_ele, sizeof(int) * m->NR);
  memcpy(ryr_jsr, m->ryr_jsr, sizeof(int) * m->NR);
  memcpy(ryr_nb, m->ryr_nb, sizeof(int) * 4 * m->NR);
  memcpy(lcc_ele, m->lcc_ele, sizeof(int) * m->NL);
}

/* ResetDefaultGridStates (cpu/InitFuncs.cpp:890-955). */
void or_initial_states(const or_mesh* m, const double* R, double* S) {
  int N = m->N, j;
  double ca0 = R[OR_C_0_CA], ca0_jsr = R[OR_C_0_CA_JSR], Kd;
  double c_trpn, c_csqn, c_atp, c_cmdn, c_dye;
  Kd = R[OR_K_OFF_TRPN] / R[OR_K_ON_TRPN];
  c_trpn = ca0 * R[OR_B_TOT_TRPN] / (Kd + ca0);
  Kd = R[OR_K_OFF_CSQN] / R[OR_K_ON_CSQN];
  c_csqn = ca0_jsr * R[OR_B_T_JSR] / (Kd + ca0_jsr);
  Kd = R[OR_K_OFF_ATP] / R[OR_K_ON_ATP];
  c_atp = ca0 * R[OR_B_TOT_ATP] / (Kd + ca0);
  Kd = R[OR_K_OFF_CMDN] / R[OR_K_ON_CMDN];
  c_cmdn = ca0 * R[OR_B_TOT_CMDN] / (Kd + ca0);
  Kd = R[OR_K_OFF_DYE] / R[OR_K_ON_DYE];
  c_dye = ca0 * R[OR_B_TOT_DYE] / (Kd + ca0);
  for (j = 0; j < N; ++j) {
    if (m->domain[j] == 0) {
      S[S_CA * N + j] = ca0;
      S[S_TRPN * N + j] = c_trpn * m->tropc[j];
      S[S_ATP * N + j] = c_atp;
      S[S_CMDN * N + j] = c_cmdn;
      S[S_DYE * N + j] = c_dye;
      S[S_CSQN * N + j] = 0.0;
    } else {
      S[S_CA * N + j] = ca0_jsr;
      S[S_TRPN * N + j] = 0;
      S[S_CSQN * N + j] = c_csqn;
      S[S_ATP * N + j] = 0;
      S[S_CMDN * N + j] = 0;
      S[S_DYE * N + j] = 0;
    }
  }
}

/* ExplicitStep (cpu/RunSimulation.cpp:591-647), gating excluded. */
void or_explicit_step(const or_mesh* m, const double* R, const double* G, double* S, const int* ryr,
                      const int* lcc, const int* lccv) {
  int N = m->N, j, i;
  double* buf;
  const double* gca = S + S_CA * N;
  if (!m->scratch) ((or_mesh*)m)->scratch = malloc(sizeof(double) * 6 * N);
  buf = m->scratch;
  /* UpdateReactionTerms (:25-125) */
  for (j = 0; j < N; ++j) {
    double c_ca = S[S_CA * N + j], r_net, c_b;
    double a0 = m->aij[5 * j], a1 = m->aij[5 * j + 1], a2 = m->aij[5 * j + 2], a3 = m->aij[5 * j + 3],
           a4 = m->aij[5 * j + 4];
    int n1 = m->nij[4 * j], n2 = m->nij[4 * j + 1], n3 = m->nij[4 * j + 2], n4 = m->nij[4 * j + 3];
    const double *Ca = S + S_CA * N, *Dy = S + S_DYE * N, *At = S + S_ATP * N, *Cm = S + S_CMDN * N;
    buf[S_TRPN * N + j] = 0;
    buf[S_CSQN * N + j] = 0;
    buf[S_CA * N + j] = R[OR_D_CA] * (c_ca * a0 + Ca[n1] * a1 + Ca[n2] * a2 + Ca[n3] * a3 + Ca[n4] * a4) +
                        m->br[S_CA * N + j];
    buf[S_DYE * N + j] = R[OR_D_DYE] * (Dy[j] * a0 + Dy[n1] * a1 + Dy[n2] * a2 + Dy[n3] * a3 + Dy[n4] * a4) +
                         m->br[S_DYE * N + j];
    buf[S_ATP * N + j] = R[OR_D_ATP] * (At[j] * a0 + At[n1] * a1 + At[n2] * a2 + At[n3] * a3 + At[n4] * a4) +
                         m->br[S_ATP * N + j];
    buf[S_CMDN * N + j] =
        R[OR_D_CMDN] * (Cm[j] * a0 + Cm[n1] * a1 + Cm[n2] * a2 + Cm[n3] * a3 + Cm[n4] * a4) +
        m->br[S_CMDN * N + j];
    if (m->domain[j] == 0) {
      if (m->tropc[j]) {
        c_b = S[S_TRPN * N + j];
        r_net = R[OR_K_ON_TRPN] * (R[OR_B_TOT_TRPN] - c_b) * c_ca - R[OR_K_OFF_TRPN] * c_b;
        buf[S_CA * N + j] += -r_net;
        buf[S_TRPN * N + j] = r_net;
        {
          double K_i = c_ca / R[OR_K_D_i];
          double K_sr, D_cycle, v_cycle, d_ca;
          K_i = K_i * K_i;
          K_sr = G[1] / R[OR_K_D_SR];
          K_sr = K_sr * K_sr;
          D_cycle = 0.104217 + 17.923 * K_sr + K_i * (1.75583e6 + K_sr * 7.61673e6) +
                    K_i * K_i * (6.08463e11 + K_sr * 4.50544e11);
          v_cycle = (K_i * K_i * 3.24873e12 + K_i * (9.17846e6 - 11478.2 * K_sr) - 0.329904 * K_sr) / D_cycle;
          d_ca = (2e-3) * v_cycle * R[OR_A_P];
          buf[S_CA * N + j] -= d_ca;
        }
      }
      c_b = S[S_DYE * N + j];
      r_net = R[OR_K_ON_DYE] * (R[OR_B_TOT_DYE] - c_b) * c_ca - R[OR_K_OFF_DYE] * c_b;
      buf[S_CA * N + j] += -r_net;
      buf[S_DYE * N + j] += r_net;
      c_b = S[S_ATP * N + j];
      r_net = R[OR_K_ON_ATP] * (R[OR_B_TOT_ATP] - c_b) * c_ca - R[OR_K_OFF_ATP] * c_b;
      buf[S_CA * N + j] += -r_net;
      buf[S_ATP * N + j] += r_net;
      c_b = S[S_CMDN * N + j];
      r_net = R[OR_K_ON_CMDN] * (R[OR_B_TOT_CMDN] - c_b) * c_ca - R[OR_K_OFF_CMDN] * c_b;
      buf[S_CA * N + j] += -r_net;
      buf[S_CMDN * N + j] += r_net;
    } else {
      c_b = S[S_CSQN * N + j];
      r_net = R[OR_K_ON_CSQN] * (R[OR_B_T_JSR] - c_b) * c_ca - R[OR_K_OFF_CSQN] * c_b;
      buf[S_CA * N + j] += -r_net;
      buf[S_CSQN * N + j] = r_net;
      buf[S_CA * N + j] += (G[1] - c_ca) * R[OR_V_REFILL];
    }
  }
  /* UpdateRyRFlux (:127-141) */
  for (i = 0; i < m->NR; ++i) {
    if (ryr[i]) {
      double J = R[OR_V_RYR] * (gca[m->ryr_jsr[i]] - gca[m->ryr_ele[i]]) * R[OR_V_CELL];
      buf[S_CA * N + m->ryr_ele[i]] += J / m->V0[m->ryr_ele[i]];
      buf[S_CA * N + m->ryr_jsr[i]] -= J / m->V0[m->ryr_jsr[i]];
    }
  }
  /* UpdateLCCFlux (:143-164) */
  for (i = 0; i < m->NL; ++i) {
    if ((lcc[i] == 6 || lcc[i] == 12) && lccv[i] == 2) {
      const double P_CaL = (9.13e-13) * (1e12) * (1e-3);
      const double F = 96.5;
      const double RT = 310 * 8.314;
      const double F_over_RT = F / RT;
      double V = G[0];
      double CA_DYAD = gca[m->lcc_ele[i]];
      double J_lcc;
      if (fabs(V) < 1e-6) V = 1e-6;
      J_lcc = -P_CaL * V * (2 * F_over_RT) * (CA_DYAD * exp(2 * V * F_over_RT) - 0.34 * R[OR_CA_0]) /
              (exp(2 * V * F_over_RT) - 1) / m->V0[m->lcc_ele[i]];
      buf[S_CA * N + m->lcc_ele[i]] += J_lcc;
    }
  }
  /* UpdateFastBuffer (:15-22) */
  for (j = 0; j < N; ++j) {
    double btothi = m->TT[j] * R[OR_B_TOT_SL_HI] / (m->V0[j] * (1e-15));
    double btotlo = m->TT[j] * R[OR_B_TOT_SL_LO] / (m->V0[j] * (1e-15));
    double kh = R[OR_K_D_SL_HI], kl = R[OR_K_D_SL_LO], c = gca[j];
    double B = 1 + (btothi * kh / ((kh + c) * (kh + c))) + (btotlo * kl / ((kl + c) * (kl + c)));
    buf[S_CA * N + j] /= B;
  }
  /* Euler (:640-644) */
  {
    double dt = R[OR_T_STEP];
    for (i = 0; i < 6; ++i)
      for (j = 0; j < N; ++j) S[i * N + j] += buf[i * N + j] * dt;
  }
}

/* ---- reference-mode gating (cpu/RunSimulation.cpp:166-400) -------------- */
static void ref_gating(const or_mesh* m, const double* R, double V, const double* ca, int* ryr, int* lcc,
                       int* lccv, double* res) {
  double dt = R[OR_T_STEP];
  int idx;
  for (idx = 0; idx < m->NR; ++idx) {
    int No = 0, Nc = 0, i;
    double X, rate, ca_ss = ca[m->ryr_ele[idx]];
    for (i = 0; i < 4; ++i)
      if (m->ryr_nb[idx * 4 + i] >= 0) {
        if (ryr[m->ryr_nb[idx * 4 + i]]) No++;
        else Nc++;
      }
    if (ryr[idx]) {
      X = exp(0.5 * R[OR_RYR_A_STAR] * (No * R[OR_RYR_EPS_OO] - Nc * R[OR_RYR_EPS_CC]));
      rate = X * R[OR_RYR_K_MINUS];
    } else {
      double phi = (1.0 - pow(1000.0 / R[OR_RYR_PHI_B], R[OR_RYR_PHI_M])) +
                   pow(ca[m->ryr_jsr[idx]] / R[OR_RYR_PHI_B], R[OR_RYR_PHI_M]);
      X = exp(0.5 * R[OR_RYR_A_STAR] * (Nc * R[OR_RYR_EPS_CC] - No * R[OR_RYR_EPS_OO]));
      rate = X * phi * R[OR_RYR_K_PLUS] * pow(ca_ss, R[OR_RYR_ETA]);
    }
    res[idx] += rate * dt;
    if (res[idx] > 0) {
      double runif = ((double)rand()) / ((double)RAND_MAX);
      res[idx] = log(runif);
      ryr[idx] = ryr[idx] == 1 ? 0 : 1;
    }
  }
  for (idx = 0; idx < m->NL; ++idx) {
    const double fL = 0.85, gL = 2.0, fLprime = 0.005, gLprime = 7.0, bL = 1.9356;
    const double bL2 = bL * bL, bL3 = bL * bL * bL, bL4 = bL * bL * bL * bL;
    const double aL = 2.0, aL2 = aL * aL, aL3 = aL * aL * aL, aL4 = aL * aL * aL * aL;
    const double omega = 0.83 * 2.0 * 1.3 * 0.01;
    const double alphacf = 4.0 * 1.2 * 0.416, betacf = 4.0 * 0.45 * 0.049;
    const double gammacf = 0.83 * 1.9 * 1.3 * 0.31 * 7.5 * 0.09233 / 1000.0;
    const double yCa_frac = 0.4;
    double ca_ss = ca[m->lcc_ele[idx]];
    double alpha = alphacf * exp(0.012 * (V - 35.0)), beta = betacf * exp(-0.05 * (V - 35.0));
    double alpha_prime = aL * alpha, beta_prime = beta / bL, gamma_rate = gammacf * ca_ss;
    int i_lcc = idx + m->NR, s = lcc[idx], tg[3] = {0, 0, 0}, vs;
    double tr[3] = {0, 0, 0}, lccv_rate, yCa_inf, tau_yCa;
    switch (s) {
      case 1: tr[0] = 4.0 * alpha; tr[1] = gamma_rate; tg[0] = 2; tg[1] = 7; break;
      case 2: tr[0] = beta; tr[1] = 3.0 * alpha; tr[2] = aL * gamma_rate; tg[0] = 1; tg[1] = 3; tg[2] = 8; break;
      case 3: tr[0] = 2.0 * beta; tr[1] = 2.0 * alpha; tr[2] = aL2 * gamma_rate; tg[0] = 2; tg[1] = 4; tg[2] = 9; break;
      case 4: tr[0] = 3.0 * beta; tr[1] = alpha; tr[2] = aL3 * gamma_rate; tg[0] = 3; tg[1] = 5; tg[2] = 10; break;
      case 5: tr[0] = 4.0 * beta; tr[1] = fL; tr[2] = aL4 * gamma_rate; tg[0] = 4; tg[1] = 6; tg[2] = 11; break;
      case 6: tr[0] = gL; tg[0] = 5; break;
      case 7: tr[0] = omega; tr[1] = 4.0 * alpha_prime; tg[0] = 1; tg[1] = 8; break;
      case 8: tr[0] = beta_prime; tr[1] = omega / bL; tr[2] = 3.0 * alpha_prime; tg[0] = 7; tg[1] = 2; tg[2] = 9; break;
      case 9: tr[0] = 2.0 * beta_prime; tr[1] = omega / bL2; tr[2] = 2.0 * alpha_prime; tg[0] = 8; tg[1] = 3; tg[2] = 10; break;
      case 10: tr[0] = 3.0 * beta_prime; tr[1] = omega / bL3; tr[2] = alpha_prime; tg[0] = 9; tg[1] = 4; tg[2] = 11; break;
      case 11: tr[0] = 4.0 * beta_prime; tr[1] = omega / bL4; tr[2] = fLprime; tg[0] = 10; tg[1] = 5; tg[2] = 12; break;
      case 12: tr[0] = gLprime; tg[0] = 11; break;
      default: break;
    }
    vs = lccv[idx];
    yCa_inf = yCa_frac / (1.0 + exp((V + 12.5) / 5.0)) + (1.0 - yCa_frac);
    tau_yCa = 60.0 + 340.0 / (1.0 + exp((V + 30.0) / 12.0));
    lccv_rate = (vs == 1) ? yCa_inf / tau_yCa : (1.0 - yCa_inf) / tau_yCa;
    res[i_lcc] += (tr[0] + tr[1] + tr[2] + lccv_rate) * dt;
    if (res[i_lcc] > 0) {
      double runif = ((double)rand()) / ((double)RAND_MAX);
      res[i_lcc] = log(runif);
      runif = (((double)rand()) / ((double)RAND_MAX)) * (tr[0] + tr[1] + tr[2] + lccv_rate);
      if (runif < tr[0]) lcc[idx] = tg[0];
      else if (runif < tr[0] + tr[1]) lcc[idx] = tg[1];
      else if (runif < tr[0] + tr[1] + tr[2]) lcc[idx] = tg[2];
      else lccv[idx] = (vs == 1) ? 2 : 1;
    }
  }
}

/* ---- PHILOX mode: the GPU's arithmetic, restated -------------------------- */
void or_philox4x32_10(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  int r;
  for (r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}
static double u01(uint32_t hi, uint32_t lo) {
  uint64_t k = ((uint64_t)hi << 20) | (uint64_t)(lo >> 12);
  return ((double)k + 0.5) * 2.220446049250313080847263336181640625e-16;
}
static void draw2(uint64_t seed, uint32_t ch, uint64_t step, uint32_t stream, double* u0, double* u1) {
  uint32_t c[4], o[4];
  c[0] = (uint32_t)step;
  c[1] = (uint32_t)(step >> 32);
  c[2] = ch;
  c[3] = stream;
  or_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32), o);
  *u0 = u01(o[0], o[1]);
  *u1 = u01(o[2], o[3]);
}
static float f_of(uint32_t b) {
  float f;
  memcpy(&f, &b, 4);
  return f;
}
static uint32_t b_of(float f) {
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
}
/* natural log: x = m 2^e, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1)) */
float or_logf(float x) {
  uint32_t b;
  int e;
  float m, s, s2, p, fe;
  if (!(x > 1.17549435e-38f)) return -1e30f;
  b = b_of(x);
  e = (int)((b >> 23) & 0xff) - 127;
  m = f_of((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e += 1;
  }
  s = (m - 1.0f) / (m + 1.0f);
  s2 = s * s;
  p = 0.0909090909f;
  p = fmaf(p, s2, 0.111111111f);
  p = fmaf(p, s2, 0.142857143f);
  p = fmaf(p, s2, 0.2f);
  p = fmaf(p, s2, 0.333333333f);
  p = fmaf(p, s2, 1.0f);
  fe = (float)e;
  return fmaf(fe, 0.693145752f, fmaf(fe, 1.42860677e-06f, (2.0f * s) * p));
}
/* 2^y: y = k + f, |f| <= 1/2, e^(f ln 2) by its Taylor polynomial */
float or_exp2f(float y) {
  int k;
  float f, t, p;
  if (y > 127.0f) y = 127.0f;
  if (y < -126.0f) y = -126.0f;
  k = (int)rintf(y);
  f = y - (float)k;
  t = f * 0.693147181f;
  p = 2.48015873e-05f;
  p = fmaf(p, t, 1.98412698e-04f);
  p = fmaf(p, t, 1.38888889e-03f);
  p = fmaf(p, t, 8.33333333e-03f);
  p = fmaf(p, t, 4.16666667e-02f);
  p = fmaf(p, t, 1.66666667e-01f);
  p = fmaf(p, t, 0.5f);
  p = fmaf(p, t, 1.0f);
  p = fmaf(p, t, 1.0f);
  return p * f_of((uint32_t)(k + 127) << 23);
}
static float or_powf(float x, float a) { return or_exp2f(a * (or_logf(x) * 1.44269504f)); }
double or_log(double x) {
  uint64_t b;
  int e;
  double m, s, s2, p;
  if (!(x > 2.2250738585072014e-308)) return -1e300;
  memcpy(&b, &x, 8);
  e = (int)((b >> 52) & 0x7ff) - 1023;
  b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
  memcpy(&m, &b, 8);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  s = (m - 1.0) / (m + 1.0);
  s2 = s * s;
  p = 1.0 / 23.0;
  p = fma(p, s2, 1.0 / 21.0);
  p = fma(p, s2, 1.0 / 19.0);
  p = fma(p, s2, 1.0 / 17.0);
  p = fma(p, s2, 1.0 / 15.0);
  p = fma(p, s2, 1.0 / 13.0);
  p = fma(p, s2, 1.0 / 11.0);
  p = fma(p, s2, 1.0 / 9.0);
  p = fma(p, s2, 1.0 / 7.0);
  p = fma(p, s2, 1.0 / 5.0);
  p = fma(p, s2, 1.0 / 3.0);
  p = fma(p, s2, 1.0);
  return fma((double)e, 0.6931471803691238, fma((double)e, 1.9082149292705877e-10, (2.0 * s) * p));
}

typedef struct {
  float kplus, kminus, eta, phi0, inv_kphi, phin, astar_half, eps_cc, eps_oo;
  float alpha, beta, gamma_cf, v_in, v_ac;
  double dt;
} or_gc;

static void make_gc(const double* R, double V, or_gc* g) {
  const double alphacf = 4.0 * 1.2 * 0.416, betacf = 4.0 * 0.45 * 0.049;
  const double gammacf = 0.83 * 1.9 * 1.3 * 0.31 * 7.5 * 0.09233 / 1000.0;
  double yinf = 0.4 / (1.0 + exp((V + 12.5) / 5.0)) + (1.0 - 0.4);
  double tau = 60.0 + 340.0 / (1.0 + exp((V + 30.0) / 12.0));
  g->kplus = (float)R[OR_RYR_K_PLUS];
  g->kminus = (float)R[OR_RYR_K_MINUS];
  g->eta = (float)R[OR_RYR_ETA];
  g->phi0 = (float)(1.0 - pow(1000.0 / R[OR_RYR_PHI_B], R[OR_RYR_PHI_M]));
  g->inv_kphi = (float)(1.0 / R[OR_RYR_PHI_B]);
  g->phin = (float)R[OR_RYR_PHI_M];
  g->astar_half = (float)(0.5 * R[OR_RYR_A_STAR]);
  g->eps_cc = (float)R[OR_RYR_EPS_CC];
  g->eps_oo = (float)R[OR_RYR_EPS_OO];
  g->alpha = (float)(alphacf * exp(0.012 * (V - 35.0)));
  g->beta = (float)(betacf * exp(-0.05 * (V - 35.0)));
  g->gamma_cf = (float)gammacf;
  g->v_in = (float)(yinf / tau);
  g->v_ac = (float)((1.0 - yinf) / tau);
  g->dt = R[OR_T_STEP];
}

void or_gating_philox(const or_mesh* m, const double* R, double V, const double* ca, uint64_t seed,
                      int64_t step, int* ryr, int* lcc, int* lccv, double* res) {
  or_gc g;
  int i, *no = malloc(sizeof(int) * (m->NR + 1)), *nc = malloc(sizeof(int) * (m->NR + 1));
  make_gc(R, V, &g);
  /* lattice counts from the states before this update (one snapshot) */
  for (i = 0; i < m->NR; ++i) {
    int q;
    no[i] = nc[i] = 0;
    for (q = 0; q < 4; ++q) {
      int j = m->ryr_nb[4 * i + q];
      if (j >= 0) {
        if (ryr[j]) no[i]++;
        else nc[i]++;
      }
    }
  }
  for (i = 0; i < m->NR; ++i) {
    float css = (float)ca[m->ryr_ele[i]], cj = (float)ca[m->ryr_jsr[i]], rate;
    double r;
    if (ryr[i]) {
      float X = 1.0f;
      if (g.astar_half != 0.0f)
        X = or_exp2f((g.astar_half * ((float)no[i] * g.eps_oo - (float)nc[i] * g.eps_cc)) * 1.44269504f);
      rate = X * g.kminus;
    } else {
      float phi = g.phi0 + or_powf(cj * g.inv_kphi, g.phin), X = 1.0f;
      if (g.astar_half != 0.0f)
        X = or_exp2f((g.astar_half * ((float)nc[i] * g.eps_cc - (float)no[i] * g.eps_oo)) * 1.44269504f);
      rate = ((X * phi) * g.kplus) * or_powf(css, g.eta);
    }
    r = res[i] + (double)rate * g.dt;
    if (r > 0.0) {
      double u0, u1;
      draw2(seed, (uint32_t)i, (uint64_t)step, 0u, &u0, &u1);
      r = or_log(u0);
      ryr[i] = !ryr[i];
    }
    res[i] = r;
  }
  for (i = 0; i < m->NL; ++i) {
    const float fL = 0.85f, gL = 2.0f, fLp = 0.005f, gLp = 7.0f, bL = 1.9356f, aL = 2.0f;
    const float omega = 0.83f * 2.0f * 1.3f * 0.01f;
    float bL2 = bL * bL, bL3 = bL2 * bL, bL4 = bL3 * bL, aL2 = aL * aL, aL3 = aL2 * aL, aL4 = aL3 * aL;
    float css = (float)ca[m->lcc_ele[i]];
    float a = g.alpha, b = g.beta, ap = aL * a, bp = b / bL, gam = g.gamma_cf * css;
    float tr[3] = {0, 0, 0}, vr, tot;
    int tg[3] = {0, 0, 0};
    double r;
    switch (lcc[i]) {
      case 1: tr[0] = 4.0f * a; tr[1] = gam; tg[0] = 2; tg[1] = 7; break;
      case 2: tr[0] = b; tr[1] = 3.0f * a; tr[2] = aL * gam; tg[0] = 1; tg[1] = 3; tg[2] = 8; break;
      case 3: tr[0] = 2.0f * b; tr[1] = 2.0f * a; tr[2] = aL2 * gam; tg[0] = 2; tg[1] = 4; tg[2] = 9; break;
      case 4: tr[0] = 3.0f * b; tr[1] = a; tr[2] = aL3 * gam; tg[0] = 3; tg[1] = 5; tg[2] = 10; break;
      case 5: tr[0] = 4.0f * b; tr[1] = fL; tr[2] = aL4 * gam; tg[0] = 4; tg[1] = 6; tg[2] = 11; break;
      case 6: tr[0] = gL; tg[0] = 5; break;
      case 7: tr[0] = omega; tr[1] = 4.0f * ap; tg[0] = 1; tg[1] = 8; break;
      case 8: tr[0] = bp; tr[1] = omega / bL; tr[2] = 3.0f * ap; tg[0] = 7; tg[1] = 2; tg[2] = 9; break;
      case 9: tr[0] = 2.0f * bp; tr[1] = omega / bL2; tr[2] = 2.0f * ap; tg[0] = 8; tg[1] = 3; tg[2] = 10; break;
      case 10: tr[0] = 3.0f * bp; tr[1] = omega / bL3; tr[2] = ap; tg[0] = 9; tg[1] = 4; tg[2] = 11; break;
      case 11: tr[0] = 4.0f * bp; tr[1] = omega / bL4; tr[2] = fLp; tg[0] = 10; tg[1] = 5; tg[2] = 12; break;
      case 12: tr[0] = gLp; tg[0] = 11; break;
      default: break;
    }
    vr = (lccv[i] == 1) ? g.v_in : g.v_ac;
    tot = ((tr[0] + tr[1]) + tr[2]) + vr;
    r = res[m->NR + i] + (double)tot * g.dt;
    if (r > 0.0) {
      double u0, u1;
      float pick, c1, c2;
      draw2(seed, (uint32_t)(m->NR + i), (uint64_t)step, 0u, &u0, &u1);
      r = or_log(u0);
      pick = (float)u1 * tot;
      c1 = tr[0] + tr[1];
      c2 = c1 + tr[2];
      if (pick < tr[0]) lcc[i] = tg[0];
      else if (pick < c1) lcc[i] = tg[1];
      else if (pick < c2) lcc[i] = tg[2];
      else lccv[i] = (lccv[i] == 1) ? 2 : 1;
    }
    res[m->NR + i] = r;
  }
  free(no);
  free(nc);
}

void or_steps_philox(const or_mesh* m, const double* R, const double* G, double* S, uint64_t seed,
                     int64_t step0, int64_t n, int* ryr, int* lcc, int* lccv, double* res) {
  int64_t s;
  for (s = 0; s < n; ++s) {
    or_explicit_step(m, R, G, S, ryr, lcc, lccv);
    or_gating_philox(m, R, G[0], S, seed, step0 + s, ryr, lcc, lccv, res);
  }
}

static double philox_protocol_u(uint64_t seed, uint32_t k) {
  double u0, u1;
  draw2(seed, 0xFFFFFF00u + k, 0xFFFFFFFFFFFFFFFFull, 2u, &u0, &u1);
  return u0;
}

/* the initial opening rule of cpu/main.cpp:217-250, with OpenRandomRyR
 * (cpu/InitFuncs.cpp:1420-1475) drawing its uniform from `u` */
static void open_initial(const or_mesh* m, const int* I, const double* R, const double* S, int* ryr,
                         int* lcc, double u) {
  if (I[OI_FLAG_LCC]) {
    lcc[I[OI_LCC_INDEX]] = 6;
  } else if (I[OI_FLAG_V_CLAMP]) {
  } else if (I[OI_INIT_RYR] != -1) {
    ryr[I[OI_INIT_RYR]] = 1;
  } else {
    int i, pick = 0;
    double tot = 0, sum = 0, r;
    double* rate = malloc(sizeof(double) * m->NR);
    for (i = 0; i < m->NR; ++i) {
      int No = 0, Nc = 0, q;
      double X, phi, ca_ss = S[S_CA * m->N + m->ryr_ele[i]];
      for (q = 0; q < 4; ++q)
        if (m->ryr_nb[i * 4 + q] >= 0) {
          if (ryr[m->ryr_nb[i * 4 + q]]) No++;
          else Nc++;
        }
      if (ryr[i]) {
        X = exp(0.5 * R[OR_RYR_A_STAR] * (No * R[OR_RYR_EPS_OO] - Nc * R[OR_RYR_EPS_CC]));
        rate[i] = X * R[OR_RYR_K_MINUS];
      } else {
        phi = R[OR_RYR_PHI_M] * S[S_CA * m->N + m->ryr_jsr[i]] + R[OR_RYR_PHI_B];
        X = exp(0.5 * R[OR_RYR_A_STAR] * (Nc * R[OR_RYR_EPS_CC] - No * R[OR_RYR_EPS_OO]));
        rate[i] = X * phi * R[OR_RYR_K_PLUS] * pow(ca_ss, R[OR_RYR_ETA]);
      }
      tot += rate[i];
    }
    r = tot * u;
    for (i = 0; i < m->NR; ++i) {
      sum += rate[i];
      if (sum >= r) {
        pick = i;
        break;
      }
    }
    ryr[pick] = 1;
    free(rate);
  }
}

void or_reset_philox(const or_mesh* m, const int* I, const double* R, uint64_t seed, double* S, int* ryr,
                     int* lcc, int* lccv, double* res, int64_t* lcc_close_step) {
  int i;
  or_initial_states(m, R, S);
  for (i = 0; i < m->NR; ++i) ryr[i] = 0;
  for (i = 0; i < m->NL; ++i) {
    lcc[i] = 1;
    lccv[i] = 2;
  }
  open_initial(m, I, R, S, ryr, lcc, philox_protocol_u(seed, 1));
  for (i = 0; i < m->NR + m->NL; ++i) {
    double u0, u1;
    draw2(seed, (uint32_t)i, 0xFFFFFFFFFFFFFFFFull, 2u, &u0, &u1);
    res[i] = or_log(u0);
  }
  *lcc_close_step = -1;
  if (I[OI_FLAG_LCC]) {
    double T = -R[OR_LCC_DURATION] * or_log(philox_protocol_u(seed, 0)), t = 0;
    int64_t n = 0;
    while (t <= R[OR_T_FINAL]) {
      if (t >= T) break;
      t += R[OR_T_STEP];
      ++n;
    }
    *lcc_close_step = n;
  }
}

/* WriteToStateFiles (cpu/OutputFuncs.cpp:241-350) */
static void states_row(const or_mesh* m, const int* I, const double* R, const double* S, const int* ryr,
                       const int* lcc, const int* lccv, double V, double t, float* row) {
  const double* ca = S;
  int k = 0, i, n_open = 0, n_lcc = 0;
  double i_ryr = 0, i_lcc = 0, mean_sr = 0, mean_i = 0;
  const double P_CaL = (9.13e-13) * (1e12) * (1e-3);
  const double F = 96.5;
  const double RT = 310 * 8.314;
  const double F_over_RT = F / RT;
  row[k++] = (float)t;
  for (i = 0; i < m->NR; ++i) {
    double CaJSR = ca[m->ryr_jsr[i]], CaSS = ca[m->ryr_ele[i]];
    i_ryr += ryr[i] * R[OR_V_RYR] * (CaJSR - CaSS) * (R[OR_V_CELL]) * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_ryr;
  for (i = 0; i < m->NR; ++i) n_open += ryr[i];
  row[k++] = (float)n_open;
  for (i = 0; i < m->NL; ++i)
    if (lccv[i] == 2 && (lcc[i] == 6 || lcc[i] == 12)) n_lcc++;
  row[k++] = (float)n_lcc;
  if (fabs(V) < 1e-6) V = 1e-6;
  for (i = 0; i < m->NL; ++i) {
    double CA_DYAD = ca[m->lcc_ele[i]];
    if ((lcc[i] == 6 || lcc[i] == 12) && lccv[i] == 2)
      i_lcc += -P_CaL * V * (2 * F_over_RT) * (CA_DYAD * exp(2 * V * F_over_RT) - 0.34 * R[OR_CA_0]) /
               (exp(2 * V * F_over_RT) - 1) * 96485 * 2 * (1e-6);
  }
  row[k++] = (float)i_lcc;
  for (i = 0; i < m->NR; ++i) mean_sr += ca[m->ryr_jsr[i]];
  mean_sr /= m->NR;
  row[k++] = (float)mean_sr;
  for (i = 0; i < m->NR; ++i) mean_i += ca[m->ryr_ele[i]];
  mean_i /= m->NR;
  row[k++] = (float)mean_i;
  if (I[OI_FLAG_RYR_OUT])
    for (i = 0; i < m->NR; ++i) row[k++] = (float)ryr[i];
}

/* RunSimulation (cpu/RunSimulation.cpp:402-589) */
int64_t or_run_simulation(const or_mesh* m, const int* I, const double* R, int mode, uint64_t seed_or_rank,
                          int index, float* rows, int64_t row_cap, int row_w, double* S_out, double* t_end,
                          int64_t* n_steps) {
  int N = m->N, NR = m->NR, NL = m->NL, NCH = m->NR + m->NL, i;
  double* S = malloc(sizeof(double) * 6 * N);
  int *ryr = calloc(NR + 1, sizeof(int)), *lcc = malloc(sizeof(int) * (NL + 1)),
      *lccv = malloc(sizeof(int) * (NL + 1));
  double* res = malloc(sizeof(double) * (NCH + 1));
  double t = 0, dt = R[OR_T_STEP], dt_last = 0, G[2], ca_ss_max = 0, T_LCC_Close = 0;
  int64_t nrows = 0, n = 0, lcc_close_step = -1;
  int N_RyR_Open = 0, bLCC_Open;
  G[0] = R[OR_DEFAULT_VM];
  G[1] = R[OR_DEFAULT_CA_NSR];
  if (mode == OR_RNG_REFERENCE) {
    int seed;
    or_initial_states(m, R, S);
    for (i = 0; i < NL; ++i) {
      lcc[i] = 1;
      lccv[i] = 2;
    }
    /* cpu/main.cpp:217-250; OpenRandomRyR reseeds and draws one rand() */
    if (!I[OI_FLAG_LCC] && !I[OI_FLAG_V_CLAMP] && I[OI_INIT_RYR] == -1) {
      int sd = 93843 + I[OI_RAND_SEED_0] + (int)seed_or_rank * I[OI_RAND_ADD_A] + index * I[OI_RAND_ADD_B];
      if (I[OI_FLAG_CLOCK_SEED]) sd += (int)time(NULL);
      srand(sd);
      open_initial(m, I, R, S, ryr, lcc, ((double)rand()) / ((double)RAND_MAX));
    } else {
      open_initial(m, I, R, S, ryr, lcc, 0.0);
    }
    if (nrows < row_cap) states_row(m, I, R, S, ryr, lcc, lccv, G[0], t, rows + nrows * row_w), ++nrows;
    for (i = 0; i < NR; ++i) N_RyR_Open += ryr[i];
    seed = 93843 + I[OI_RAND_SEED_0] + (int)seed_or_rank * I[OI_RAND_ADD_A] + index * I[OI_RAND_ADD_B];
    if (I[OI_FLAG_CLOCK_SEED]) seed += (int)time(NULL);
    srand(seed);
    for (i = 0; i < NCH; ++i) res[i] = log(((double)rand()) / ((double)RAND_MAX));
    T_LCC_Close = -R[OR_LCC_DURATION] * log(((double)rand()) / ((double)RAND_MAX));
  } else {
    or_reset_philox(m, I, R, seed_or_rank, S, ryr, lcc, lccv, res, &lcc_close_step);
    if (nrows < row_cap) states_row(m, I, R, S, ryr, lcc, lccv, G[0], t, rows + nrows * row_w), ++nrows;
    for (i = 0; i < NR; ++i) N_RyR_Open += ryr[i];
  }
  bLCC_Open = I[OI_FLAG_LCC];
  while (t <= R[OR_T_FINAL] &&
         (!I[OI_FLAG_FIDELITY_SIM] ||
          ((bLCC_Open || N_RyR_Open > 0 || ca_ss_max > R[OR_C_MIN]) && N_RyR_Open < I[OI_N_RYR_FIDELITY]))) {
    int lcc_event = (mode == OR_RNG_REFERENCE) ? (t >= T_LCC_Close) : (lcc_close_step >= 0 && n >= lcc_close_step);
    if (I[OI_FLAG_LCC] && bLCC_Open && lcc_event) {
      bLCC_Open = 0;
      lcc[I[OI_LCC_INDEX]] = 1;
    }
    if (I[OI_FLAG_V_CLAMP]) G[0] = (t <= R[OR_T_CLAMP]) ? R[OR_V_CLAMP] : R[OR_DEFAULT_VM];
    if (I[OI_INIT_RYR] != -1 && t < R[OR_INIT_RYR_HOLD] && !ryr[I[OI_INIT_RYR]]) ryr[I[OI_INIT_RYR]] = 1;
    if (floor(t / R[OR_STATES_INTERVAL]) > floor((t - dt_last) / R[OR_STATES_INTERVAL])) {
      N_RyR_Open = 0;
      ca_ss_max = 0;
      for (i = 0; i < NR; ++i) {
        double c = S[m->ryr_ele[i]];
        N_RyR_Open += ryr[i];
        if (c > ca_ss_max) ca_ss_max = c;
      }
      if (nrows < row_cap) states_row(m, I, R, S, ryr, lcc, lccv, G[0], t, rows + nrows * row_w), ++nrows;
    }
    or_explicit_step(m, R, G, S, ryr, lcc, lccv);
    if (!I[OI_FLAG_NO_GATING]) {
      if (mode == OR_RNG_REFERENCE) ref_gating(m, R, G[0], S, ryr, lcc, lccv, res);
      else or_gating_philox(m, R, G[0], S, seed_or_rank, n, ryr, lcc, lccv, res);
    }
    t += dt;
    dt_last = dt;
    ++n;
  }
  if (nrows < row_cap) states_row(m, I, R, S, ryr, lcc, lccv, G[0], t, rows + nrows * row_w), ++nrows;
  if (S_out) memcpy(S_out, S, sizeof(double) * 6 * N);
  if (t_end) *t_end = t;
  if (n_steps) *n_steps = n;
  free(S);
  free(ryr);
  free(lcc);
  free(lccv);
  free(res);
  return nrows;
}


/* ---- FP32 engine restated (deviation form, see k_fp32.cu's tet_update) ----
 * The GPU's FP32 engines store u = c - c_rest and evaluate each element's
 * update with the operation order below (every fused multiply-add explicit).
 * This restatement is the bit-exact CPU model of those engines. */
typedef struct {
  float D[4], kon[5], koff[5], bfree[5], c0, c0j, inv_kdi, sd0, sd1, sd2, sn1, sn0, serca_scale,
      refill_v, refill0, khi, dt, jr_scale, dc0, lccA, lccE, lccB;
  double rest_atp, rest_cmdn, rest_dye, rest_trpn, rest_csqn, rest_ca, rest_caj;
} or_k32;

static void make_k32(const double* R, double V, double nsr, or_k32* k) {
  double ca0 = R[OR_C_0_CA], ca0j = R[OR_C_0_CA_JSR], Kd, Ksr;
  double P_CaL = (9.13e-13) * (1e12) * (1e-3), F_over_RT = 96.5 / (310 * 8.314), A, E, Em1;
  const int ion[5] = {OR_K_ON_DYE, OR_K_ON_ATP, OR_K_ON_CMDN, OR_K_ON_TRPN, OR_K_ON_CSQN};
  const int ioff[5] = {OR_K_OFF_DYE, OR_K_OFF_ATP, OR_K_OFF_CMDN, OR_K_OFF_TRPN, OR_K_OFF_CSQN};
  double btot[5], brest[5];
  int q;
  Kd = R[OR_K_OFF_TRPN] / R[OR_K_ON_TRPN];
  k->rest_trpn = ca0 * R[OR_B_TOT_TRPN] / (Kd + ca0);
  Kd = R[OR_K_OFF_CSQN] / R[OR_K_ON_CSQN];
  k->rest_csqn = ca0j * R[OR_B_T_JSR] / (Kd + ca0j);
  Kd = R[OR_K_OFF_ATP] / R[OR_K_ON_ATP];
  k->rest_atp = ca0 * R[OR_B_TOT_ATP] / (Kd + ca0);
  Kd = R[OR_K_OFF_CMDN] / R[OR_K_ON_CMDN];
  k->rest_cmdn = ca0 * R[OR_B_TOT_CMDN] / (Kd + ca0);
  Kd = R[OR_K_OFF_DYE] / R[OR_K_ON_DYE];
  k->rest_dye = ca0 * R[OR_B_TOT_DYE] / (Kd + ca0);
  k->rest_ca = ca0;
  k->rest_caj = ca0j;
  btot[0] = R[OR_B_TOT_DYE];
  btot[1] = R[OR_B_TOT_ATP];
  btot[2] = R[OR_B_TOT_CMDN];
  btot[3] = R[OR_B_TOT_TRPN];
  btot[4] = R[OR_B_T_JSR];
  brest[0] = k->rest_dye;
  brest[1] = k->rest_atp;
  brest[2] = k->rest_cmdn;
  brest[3] = k->rest_trpn;
  brest[4] = k->rest_csqn;
  k->D[0] = (float)R[OR_D_CA];
  k->D[1] = (float)R[OR_D_ATP];
  k->D[2] = (float)R[OR_D_CMDN];
  k->D[3] = (float)R[OR_D_DYE];
  for (q = 0; q < 5; ++q) {
    k->kon[q] = (float)R[ion[q]];
    k->koff[q] = (float)R[ioff[q]];
    k->bfree[q] = (float)(btot[q] - brest[q]);
  }
  k->c0 = (float)ca0;
  k->c0j = (float)ca0j;
  k->inv_kdi = (float)(1.0 / R[OR_K_D_i]);
  Ksr = nsr / R[OR_K_D_SR];
  Ksr = Ksr * Ksr;
  k->sd0 = (float)(0.104217 + 17.923 * Ksr);
  k->sd1 = (float)(1.75583e6 + Ksr * 7.61673e6);
  k->sd2 = (float)(6.08463e11 + Ksr * 4.50544e11);
  k->sn1 = (float)(9.17846e6 - 11478.2 * Ksr);
  k->sn0 = (float)(0.329904 * Ksr);
  k->serca_scale = (float)(2e-3 * R[OR_A_P]);
  k->refill_v = (float)R[OR_V_REFILL];
  k->refill0 = (float)((nsr - ca0j) * R[OR_V_REFILL]);
  k->khi = (float)R[OR_K_D_SL_HI];
  k->dt = (float)R[OR_T_STEP];
  k->jr_scale = (float)(R[OR_V_RYR] * R[OR_V_CELL]);
  k->dc0 = (float)(ca0j - ca0);
  if (fabs(V) < 1e-6) V = 1e-6;
  A = -P_CaL * V * (2 * F_over_RT);
  E = exp(2 * V * F_over_RT);
  Em1 = exp(2 * V * F_over_RT) - 1;
  k->lccA = (float)(A / Em1);
  k->lccE = (float)E;
  k->lccB = (float)(0.34 * R[OR_CA_0]);
}

/* absolute (6N doubles, reference numbering) <-> deviation (4N + N floats) */
void or_fp32_to_dev(const or_mesh* m, const double* R, const double* S, float* U, float* Im) {
  or_k32 k;
  int N = m->N, j;
  make_k32(R, R[OR_DEFAULT_VM], R[OR_DEFAULT_CA_NSR], &k);
  for (j = 0; j < N; ++j) {
    int jsr = m->domain[j] == 1;
    U[4 * j + 0] = (float)(S[S_CA * N + j] - (jsr ? k.rest_caj : k.rest_ca));
    U[4 * j + 1] = (float)(S[S_ATP * N + j] - (jsr ? 0.0 : k.rest_atp));
    U[4 * j + 2] = (float)(S[S_CMDN * N + j] - (jsr ? 0.0 : k.rest_cmdn));
    U[4 * j + 3] = (float)(S[S_DYE * N + j] - (jsr ? 0.0 : k.rest_dye));
    Im[j] = jsr ? (float)(S[S_CSQN * N + j] - k.rest_csqn)
                : (float)(S[S_TRPN * N + j] - (m->tropc[j] ? k.rest_trpn : 0.0));
  }
}
void or_fp32_from_dev(const or_mesh* m, const double* R, const float* U, const float* Im, const float* CM,
                      const float* CI, double* S) {
  or_k32 k;
  int N = m->N, j;
  make_k32(R, R[OR_DEFAULT_VM], R[OR_DEFAULT_CA_NSR], &k);
  for (j = 0; j < N; ++j) {
    int jsr = m->domain[j] == 1;
    S[S_CA * N + j] = (jsr ? k.rest_caj : k.rest_ca) + ((double)U[4 * j] - (double)CM[4 * j]);
    S[S_ATP * N + j] = (jsr ? 0.0 : k.rest_atp) + ((double)U[4 * j + 1] - (double)CM[4 * j + 1]);
    S[S_CMDN * N + j] = (jsr ? 0.0 : k.rest_cmdn) + ((double)U[4 * j + 2] - (double)CM[4 * j + 2]);
    S[S_DYE * N + j] = (jsr ? 0.0 : k.rest_dye) + ((double)U[4 * j + 3] - (double)CM[4 * j + 3]);
    if (jsr) {
      S[S_CSQN * N + j] = k.rest_csqn + ((double)Im[j] - (double)CI[j]);
      S[S_TRPN * N + j] = 0.0;
    } else {
      S[S_TRPN * N + j] = (m->tropc[j] ? k.rest_trpn : 0.0) + ((double)Im[j] - (double)CI[j]);
      S[S_CSQN * N + j] = 0.0;
    }
  }
}

static void fp32_element(const or_k32* k, const float* o, float im, const float* s1, const float* s2,
                         const float* s3, const float* s4, const float* a, int jsr, int tropc, float bsl,
                         float flux, float* cm, float* ci, float* out, float* im_out) {
  float dx = a[0] * (s1[0] - o[0]), dy = a[0] * (s1[1] - o[1]), dz = a[0] * (s1[2] - o[2]),
        dw = a[0] * (s1[3] - o[3]);
  float rca, ratp, rcmdn, rdye, rim = 0.0f, u = o[0], c, rb;
  dx = fmaf(a[1], s2[0] - o[0], dx);
  dx = fmaf(a[2], s3[0] - o[0], dx);
  dx = fmaf(a[3], s4[0] - o[0], dx);
  dy = fmaf(a[1], s2[1] - o[1], dy);
  dy = fmaf(a[2], s3[1] - o[1], dy);
  dy = fmaf(a[3], s4[1] - o[1], dy);
  dz = fmaf(a[1], s2[2] - o[2], dz);
  dz = fmaf(a[2], s3[2] - o[2], dz);
  dz = fmaf(a[3], s4[2] - o[2], dz);
  dw = fmaf(a[1], s2[3] - o[3], dw);
  dw = fmaf(a[2], s3[3] - o[3], dw);
  dw = fmaf(a[3], s4[3] - o[3], dw);
  rca = k->D[0] * dx;
  ratp = k->D[1] * dy;
  rcmdn = k->D[2] * dz;
  rdye = k->D[3] * dw;
  if (!jsr) {
    c = k->c0 + u;
    if (tropc) {
      float Ki, Ki2, den, num;
      rb = fmaf(k->kon[3], fmaf(k->bfree[3], u, -im * c), -k->koff[3] * im);
      rca -= rb;
      rim = rb;
      Ki = c * k->inv_kdi;
      Ki = Ki * Ki;
      Ki2 = Ki * Ki;
      den = fmaf(Ki2, k->sd2, fmaf(Ki, k->sd1, k->sd0));
      num = fmaf(Ki2, 3.24873e12f, fmaf(Ki, k->sn1, -k->sn0));
      rca = fmaf(-k->serca_scale, num / den, rca);
    }
    rb = fmaf(k->kon[0], fmaf(k->bfree[0], u, -o[3] * c), -k->koff[0] * o[3]);
    rca -= rb;
    rdye += rb;
    rb = fmaf(k->kon[1], fmaf(k->bfree[1], u, -o[1] * c), -k->koff[1] * o[1]);
    rca -= rb;
    ratp += rb;
    rb = fmaf(k->kon[2], fmaf(k->bfree[2], u, -o[2] * c), -k->koff[2] * o[2]);
    rca -= rb;
    rcmdn += rb;
  } else {
    c = k->c0j + u;
    rb = fmaf(k->kon[4], fmaf(k->bfree[4], u, -im * c), -k->koff[4] * im);
    rca -= rb;
    rim = rb;
    rca += fmaf(-u, k->refill_v, k->refill0);
  }
  rca += flux;
  if (bsl != 0.0f) {
    float kc = k->khi + c, kc2 = kc * kc;
    rca = (rca * kc2) / (kc2 + bsl);
  }
  /* compensated (Kahan) Euler update: y = dt*r - comp; t = u + y;
   * comp = (t - u) - y */
  {
    float r4[4] = {rca, ratp, rcmdn, rdye}, y, t;
    int q;
    for (q = 0; q < 4; ++q) {
      y = fmaf(k->dt, r4[q], -cm[q]);
      t = o[q] + y;
      cm[q] = (t - o[q]) - y;
      out[q] = t;
    }
    y = fmaf(k->dt, rim, -*ci);
    t = im + y;
    *ci = (t - im) - y;
    *im_out = t;
  }
}

/* n FP32 steps (+ PHILOX gating on float Ca when `gating`), reference numbering. */
/* Compact compensation (the large-mesh form of the plain FP32 engine,
 * srs_gb300/csrc/srs_comp.h): after each update the compensation term c is
 * kept as the IEEE half of c * 2^24 (clamped to +-65504, rounded to nearest
 * even) and read back times 2^-24.  The conversion here is the compiler's
 * _Float16 (IEEE binary16, round to nearest even), independent of the
 * engine's. */
static float comp_round_trip(float c) {
  float v = c * 16777216.0f;
  _Float16 h;
  if (v == v) v = fminf(fmaxf(v, -65504.0f), 65504.0f); /* a NaN stays a NaN */
  h = (_Float16)v;
  return (float)h * (1.0f / 16777216.0f);
}

/* the round trip alone, for tests */
float or_comp_round_trip(float c) { return comp_round_trip(c); }

/* flags: bit 0 gating, bit 1 compact compensation */
void or_steps_fp32(const or_mesh* m, const double* R, const double* G, float* U, float* Im, float* CM,
                   float* CI, uint64_t seed, int64_t step0, int64_t n, int* ryr, int* lcc, int* lccv,
                   double* res, int flags) {
  const int gating = flags & 1, compact = flags & 2;
  int N = m->N, j, q, i;
  or_k32 k;
  float* U2 = malloc(sizeof(float) * 4 * N);
  float* I2 = malloc(sizeof(float) * N);
  float* a = malloc(sizeof(float) * 4 * N);
  float* bsl = malloc(sizeof(float) * N);
  float* rest = malloc(sizeof(float) * N);
  double* ca = malloc(sizeof(double) * N);
  int64_t s;
  make_k32(R, G[0], G[1], &k);
  for (j = 0; j < N; ++j) {
    double bhi = m->TT[j] * R[OR_B_TOT_SL_HI] / (m->V0[j] * (1e-15));
    for (q = 0; q < 4; ++q) a[4 * j + q] = (float)m->aij[5 * j + 1 + q];
    bsl[j] = (float)(bhi * R[OR_K_D_SL_HI]);
    rest[j] = m->domain[j] == 1 ? k.c0j : k.c0;
  }
  for (s = 0; s < n; ++s) {
    for (j = 0; j < N; ++j) {
      float flux = 0.0f;
      const int* nb = &m->nij[4 * j];
      for (i = 0; i < m->NR; ++i) {
        if (m->ryr_ele[i] == j && ryr[i]) {
          float dc = (k.dc0 + U[4 * m->ryr_jsr[i]]) - U[4 * m->ryr_ele[i]];
          flux = fmaf(k.jr_scale * dc, (float)(1.0 / m->V0[j]), flux);
        }
        if (m->ryr_jsr[i] == j && ryr[i]) {
          float dc = (k.dc0 + U[4 * m->ryr_jsr[i]]) - U[4 * m->ryr_ele[i]];
          flux = fmaf(k.jr_scale * dc, (float)(-(1.0 / m->V0[j])), flux);
        }
      }
      for (i = 0; i < m->NL; ++i)
        if (m->lcc_ele[i] == j && (lcc[i] == 6 || lcc[i] == 12) && lccv[i] == 2) {
          float c = rest[j] + U[4 * j];
          flux = fmaf(k.lccA * fmaf(c, k.lccE, -k.lccB), (float)(1.0 / m->V0[j]), flux);
        }
      fp32_element(&k, &U[4 * j], Im[j], &U[4 * nb[0]], &U[4 * nb[1]], &U[4 * nb[2]], &U[4 * nb[3]],
                   &a[4 * j], m->domain[j] == 1, m->tropc[j], bsl[j], flux, &CM[4 * j], &CI[j],
                   &U2[4 * j], &I2[j]);
      if (compact) {
        for (q = 0; q < 4; ++q) CM[4 * j + q] = comp_round_trip(CM[4 * j + q]);
        CI[j] = comp_round_trip(CI[j]);
      }
    }
    memcpy(U, U2, sizeof(float) * 4 * N);
    memcpy(Im, I2, sizeof(float) * N);
    if (gating) {
      for (j = 0; j < N; ++j) ca[j] = (double)(rest[j] + U[4 * j]);
      or_gating_philox(m, R, G[0], ca, seed, step0 + s, ryr, lcc, lccv, res);
    }
  }
  free(U2);
  free(I2);
  free(a);
  free(bsl);
  free(rest);
  free(ca);
}

/* ---- pathwise adjoint, FP64 (restatement used to check the GPU adjoint) ----
 * Forward: n steps of ExplicitStep with PHILOX gating from the given state;
 * the channel states of every step are recorded and the adjoint is taken
 * with them held fixed (pathwise sensitivity).  Loss at ticks k*te
 * (k = 1..n/te) of the bound-dye line scan F_i = pad_i + sum_j W_ij y_j:
 *   L = 1/2 sum_k sum_i (F_ki / F0_i - 1 - target_ki)^2.
 * Parameters (indices of ParamStruct::Reals) are listed in or_adj_params. */
#define OR_N_ADJ 18
const int or_adj_params[OR_N_ADJ] = {OR_D_CA, OR_D_DYE, OR_K_ON_CMDN, OR_K_OFF_CMDN,
                                     OR_K_ON_TRPN, OR_K_OFF_TRPN, OR_K_ON_CSQN, OR_K_OFF_CSQN,
                                     OR_K_ON_DYE, OR_K_OFF_DYE, OR_V_RYR, OR_A_P,
                                     OR_B_TOT_SL_HI, OR_K_D_SL_HI, OR_D_ATP, OR_D_CMDN,
                                     OR_K_ON_ATP, OR_K_OFF_ATP};

static double tick_loss(const or_mesh* m, int ns, const double* W, const double* pad, const double* F0,
                        const double* target, const double* S, double* dLdy) {
  int N = m->N, i, j;
  double L = 0;
  for (i = 0; i < ns; ++i) {
    double F = pad[i], e;
    for (j = 0; j < N; ++j) F += W[(size_t)i * N + j] * S[S_DYE * N + j];
    e = F / F0[i] - 1.0 - target[i];
    L += 0.5 * e * e;
    if (dLdy)
      for (j = 0; j < N; ++j) dLdy[j] += e * W[(size_t)i * N + j] / F0[i];
  }
  return L;
}

/* one step of the transposed linearised dynamics: out += dt * J(x)^T lam,
 * grad += dt * (dF/dtheta)(x)^T lam */
static void adj_step(const or_mesh* m, const double* R, const double* G, const double* x, const int* ryr,
                     const int* lcc, const int* lccv, const double* lam, double* out, double* grad) {
  int N = m->N, j, k, i;
  double dt = R[OR_T_STEP];
  const double *c = x + S_CA * N, *yd = x + S_DYE * N, *at = x + S_ATP * N, *cm = x + S_CMDN * N;
  const double *tr = x + S_TRPN * N, *cq = x + S_CSQN * N;
  const double P_CaL = (9.13e-13) * (1e12) * (1e-3), F_over_RT = 96.5 / (310 * 8.314);
  double V = G[0], A, E, Em1;
  double* Bv = malloc(sizeof(double) * N);
  double* Gv = malloc(sizeof(double) * N);
  if (fabs(V) < 1e-6) V = 1e-6;
  A = -P_CaL * V * (2 * F_over_RT);
  E = exp(2 * V * F_over_RT);
  Em1 = exp(2 * V * F_over_RT) - 1;
  /* pre-buffer Ca rate G and buffer factor B of every element */
  for (j = 0; j < N; ++j) {
    double Kh = R[OR_K_D_SL_HI], Kl = R[OR_K_D_SL_LO];
    double bhi = m->TT[j] * R[OR_B_TOT_SL_HI] / (m->V0[j] * (1e-15));
    double blo = m->TT[j] * R[OR_B_TOT_SL_LO] / (m->V0[j] * (1e-15));
    double g = R[OR_D_CA] * (m->aij[5 * j] * c[j]) + m->br[S_CA * N + j];
    for (k = 0; k < 4; ++k) g += R[OR_D_CA] * m->aij[5 * j + 1 + k] * c[m->nij[4 * j + k]];
    if (m->domain[j] == 0) {
      if (m->tropc[j]) {
        double Ki = c[j] / R[OR_K_D_i], Ksr = G[1] / R[OR_K_D_SR], Dc, vc;
        Ki *= Ki;
        Ksr *= Ksr;
        Dc = 0.104217 + 17.923 * Ksr + Ki * (1.75583e6 + Ksr * 7.61673e6) + Ki * Ki * (6.08463e11 + Ksr * 4.50544e11);
        vc = (Ki * Ki * 3.24873e12 + Ki * (9.17846e6 - 11478.2 * Ksr) - 0.329904 * Ksr) / Dc;
        g -= R[OR_K_ON_TRPN] * (R[OR_B_TOT_TRPN] - tr[j]) * c[j] - R[OR_K_OFF_TRPN] * tr[j];
        g -= 2e-3 * vc * R[OR_A_P];
      }
      g -= R[OR_K_ON_DYE] * (R[OR_B_TOT_DYE] - yd[j]) * c[j] - R[OR_K_OFF_DYE] * yd[j];
      g -= R[OR_K_ON_ATP] * (R[OR_B_TOT_ATP] - at[j]) * c[j] - R[OR_K_OFF_ATP] * at[j];
      g -= R[OR_K_ON_CMDN] * (R[OR_B_TOT_CMDN] - cm[j]) * c[j] - R[OR_K_OFF_CMDN] * cm[j];
    } else {
      g -= R[OR_K_ON_CSQN] * (R[OR_B_T_JSR] - cq[j]) * c[j] - R[OR_K_OFF_CSQN] * cq[j];
      g += (G[1] - c[j]) * R[OR_V_REFILL];
    }
    Gv[j] = g;
    Bv[j] = 1 + bhi * Kh / ((Kh + c[j]) * (Kh + c[j])) + blo * Kl / ((Kl + c[j]) * (Kl + c[j]));
  }
  for (i = 0; i < m->NR; ++i)
    if (ryr[i]) {
      double J = R[OR_V_RYR] * (c[m->ryr_jsr[i]] - c[m->ryr_ele[i]]) * R[OR_V_CELL];
      Gv[m->ryr_ele[i]] += J / m->V0[m->ryr_ele[i]];
      Gv[m->ryr_jsr[i]] -= J / m->V0[m->ryr_jsr[i]];
    }
  for (i = 0; i < m->NL; ++i)
    if ((lcc[i] == 6 || lcc[i] == 12) && lccv[i] == 2) {
      int e = m->lcc_ele[i];
      Gv[e] += A * (c[e] * E - 0.34 * R[OR_CA_0]) / Em1 / m->V0[e];
    }
  /* rows of J, scattered into columns */
  for (j = 0; j < N; ++j) {
    double lc = lam[S_CA * N + j], B = Bv[j], w = lc / B;
    double Kh = R[OR_K_D_SL_HI], Kl = R[OR_K_D_SL_LO];
    double bhi = m->TT[j] * R[OR_B_TOT_SL_HI] / (m->V0[j] * (1e-15));
    double blo = m->TT[j] * R[OR_B_TOT_SL_LO] / (m->V0[j] * (1e-15));
    double dB = -2 * bhi * Kh / ((Kh + c[j]) * (Kh + c[j]) * (Kh + c[j])) -
                2 * blo * Kl / ((Kl + c[j]) * (Kl + c[j]) * (Kl + c[j]));
    double dGdc = R[OR_D_CA] * m->aij[5 * j];
    int sp;
    double Dsp[4] = {R[OR_D_DYE], R[OR_D_ATP], R[OR_D_CMDN], 0};
    int sidx[3] = {S_DYE, S_ATP, S_CMDN};
    /* Ca diffusion: d(G/B)/dc_k = D a_k / B */
    for (k = 0; k < 4; ++k) out[S_CA * N + m->nij[4 * j + k]] += dt * R[OR_D_CA] * m->aij[5 * j + 1 + k] * w;
    /* mobile buffers diffusion */
    for (sp = 0; sp < 3; ++sp) {
      double lb = lam[sidx[sp] * N + j];
      out[sidx[sp] * N + j] += dt * Dsp[sp] * m->aij[5 * j] * lb;
      for (k = 0; k < 4; ++k) out[sidx[sp] * N + m->nij[4 * j + k]] += dt * Dsp[sp] * m->aij[5 * j + 1 + k] * lb;
    }
    {
      double Lc = m->aij[5 * j] * c[j], Ly = m->aij[5 * j] * yd[j];
      double La = m->aij[5 * j] * at[j], Lm = m->aij[5 * j] * cm[j];
      for (k = 0; k < 4; ++k) {
        Lc += m->aij[5 * j + 1 + k] * c[m->nij[4 * j + k]];
        Ly += m->aij[5 * j + 1 + k] * yd[m->nij[4 * j + k]];
        La += m->aij[5 * j + 1 + k] * at[m->nij[4 * j + k]];
        Lm += m->aij[5 * j + 1 + k] * cm[m->nij[4 * j + k]];
      }
      /* boundary rates are D times a fixed source */
      if (R[OR_D_CA] != 0) Lc += m->br[S_CA * N + j] / R[OR_D_CA];
      if (R[OR_D_DYE] != 0) Ly += m->br[S_DYE * N + j] / R[OR_D_DYE];
      if (R[OR_D_ATP] != 0) La += m->br[S_ATP * N + j] / R[OR_D_ATP];
      if (R[OR_D_CMDN] != 0) Lm += m->br[S_CMDN * N + j] / R[OR_D_CMDN];
      grad[0] += dt * w * Lc;
      grad[1] += dt * lam[S_DYE * N + j] * Ly;
      grad[14] += dt * lam[S_ATP * N + j] * La;
      grad[15] += dt * lam[S_CMDN * N + j] * Lm;
    }
    /* boundary rates of the mobile buffers hold their resting values
     * c0 B/(Kd + c0), Kd = koff/kon (cpu/InitFuncs.cpp:1005-1039, restated in or_mesh_load) */
    {
      int q;
      const int sp2[3] = {S_DYE, S_CMDN, S_ATP}, kon2[3] = {OR_K_ON_DYE, OR_K_ON_CMDN, OR_K_ON_ATP},
                koff2[3] = {OR_K_OFF_DYE, OR_K_OFF_CMDN, OR_K_OFF_ATP}, g2[3] = {8, 2, 16};
      for (q = 0; q < 3; ++q) {
        double brs = m->br[sp2[q] * N + j];
        if (brs != 0) {
          double kon = R[kon2[q]], Kd = R[koff2[q]] / kon, den = Kd + R[OR_C_0_CA];
          grad[g2[q]] += dt * lam[sp2[q] * N + j] * brs * Kd / (kon * den);
          grad[g2[q] + 1] += dt * lam[sp2[q] * N + j] * brs * (-1.0 / (kon * den));
        }
      }
    }
    if (m->domain[j] == 0) {
      /* buffers: r_b = kon (B - b) c - koff b;  F_c -= r_b,  F_b += r_b */
      struct { int s, kon, koff, btot, gkon; } bf[4] = {{S_DYE, OR_K_ON_DYE, OR_K_OFF_DYE, OR_B_TOT_DYE, 8},
                                                       {S_ATP, OR_K_ON_ATP, OR_K_OFF_ATP, OR_B_TOT_ATP, 16},
                                                       {S_CMDN, OR_K_ON_CMDN, OR_K_OFF_CMDN, OR_B_TOT_CMDN, 2},
                                                       {S_TRPN, OR_K_ON_TRPN, OR_K_OFF_TRPN, OR_B_TOT_TRPN, 4}};
      int q, nb = m->tropc[j] ? 4 : 3;
      for (q = 0; q < nb; ++q) {
        double b = x[bf[q].s * N + j], kon = R[bf[q].kon], koff = R[bf[q].koff];
        double alpha = kon * (R[bf[q].btot] - b), beta = kon * c[j] + koff;
        double lb = lam[bf[q].s * N + j];
        dGdc -= alpha;
        out[bf[q].s * N + j] += dt * beta * w;    /* dF_c/db = +beta/B */
        out[bf[q].s * N + j] += dt * (-beta) * lb; /* dF_b/db = -beta */
        out[S_CA * N + j] += dt * alpha * lb;     /* dF_b/dc = alpha */
        if (bf[q].gkon >= 0) {
          double dr_kon = (R[bf[q].btot] - b) * c[j], dr_koff = -b;
          grad[bf[q].gkon] += dt * (lb - w) * dr_kon;
          grad[bf[q].gkon + 1] += dt * (lb - w) * dr_koff;
        }
      }
      if (m->tropc[j]) {
        double Kd = R[OR_K_D_i], Ki = (c[j] / Kd) * (c[j] / Kd), Ksr = (G[1] / R[OR_K_D_SR]) * (G[1] / R[OR_K_D_SR]);
        double d0 = 0.104217 + 17.923 * Ksr, d1 = 1.75583e6 + Ksr * 7.61673e6, d2 = 6.08463e11 + Ksr * 4.50544e11;
        double n1 = 9.17846e6 - 11478.2 * Ksr, n0 = 0.329904 * Ksr;
        double Dn = d0 + Ki * d1 + Ki * Ki * d2, Nn = Ki * Ki * 3.24873e12 + Ki * n1 - n0;
        double dN = 2 * Ki * 3.24873e12 + n1, dD = d1 + 2 * Ki * d2;
        double dv_dKi = (dN * Dn - Nn * dD) / (Dn * Dn), dKi_dc = 2 * c[j] / (Kd * Kd);
        dGdc -= 2e-3 * R[OR_A_P] * dv_dKi * dKi_dc;
        grad[11] += dt * w * (-2e-3 * Nn / Dn);
      }
    } else {
      double b = cq[j], kon = R[OR_K_ON_CSQN], koff = R[OR_K_OFF_CSQN];
      double alpha = kon * (R[OR_B_T_JSR] - b), beta = kon * c[j] + koff, lb = lam[S_CSQN * N + j];
      dGdc -= alpha;
      dGdc -= R[OR_V_REFILL];
      out[S_CSQN * N + j] += dt * beta * w;
      out[S_CSQN * N + j] += dt * (-beta) * lb;
      out[S_CA * N + j] += dt * alpha * lb;
      grad[6] += dt * (lb - w) * (R[OR_B_T_JSR] - b) * c[j];
      grad[7] += dt * (lb - w) * (-b);
    }
    /* element-local channel terms */
    for (i = 0; i < m->NR; ++i)
      if (ryr[i] && (m->ryr_ele[i] == j || m->ryr_jsr[i] == j)) dGdc -= R[OR_V_RYR] * R[OR_V_CELL] / m->V0[j];
    for (i = 0; i < m->NL; ++i)
      if (m->lcc_ele[i] == j && (lcc[i] == 6 || lcc[i] == 12) && lccv[i] == 2) dGdc += A * E / Em1 / m->V0[j];
    /* dF_c/dc_j = dG/dc / B - G B' / B^2 */
    out[S_CA * N + j] += dt * (dGdc / B - Gv[j] * dB / (B * B)) * lc;
    /* SL buffer capacity and affinity */
    {
      double cc = c[j];
      double dB_dBtot = (m->TT[j] / (m->V0[j] * (1e-15))) * Kh / ((Kh + cc) * (Kh + cc));
      double dB_dK = bhi * (cc - Kh) / ((Kh + cc) * (Kh + cc) * (Kh + cc));
      grad[12] += dt * lc * (-Gv[j] / (B * B)) * dB_dBtot;
      grad[13] += dt * lc * (-Gv[j] / (B * B)) * dB_dK;
    }
  }
  /* RyR cross terms and V_RYR */
  for (i = 0; i < m->NR; ++i)
    if (ryr[i]) {
      int cl = m->ryr_ele[i], js = m->ryr_jsr[i];
      double v = R[OR_V_RYR] * R[OR_V_CELL];
      double wcl = lam[S_CA * N + cl] / Bv[cl], wjs = lam[S_CA * N + js] / Bv[js];
      out[S_CA * N + js] += dt * v / m->V0[cl] * wcl; /* dF_cl/dc_js */
      out[S_CA * N + cl] += dt * v / m->V0[js] * wjs; /* dF_js/dc_cl */
      grad[10] += dt * (wcl / m->V0[cl] - wjs / m->V0[js]) * R[OR_V_CELL] * (c[js] - c[cl]);
    }
  free(Bv);
  free(Gv);
}

double or_adjoint(const or_mesh* m, const int* I, const double* R, const double* S0, const int* ryr0,
                  const int* lcc0, const int* lccv0, const double* res0, uint64_t seed, int64_t n_steps,
                  int tick_every, int ns, const double* W, const double* pad, const double* F0,
                  const double* target, double* grad, double* lam0) {
  int N = m->N, NR = m->NR, NL = m->NL, k;
  int64_t n;
  double G[2], L = 0;
  double* X = malloc(sizeof(double) * 6 * N * (size_t)(n_steps + 1));
  int* RY = malloc(sizeof(int) * NR * (size_t)(n_steps + 1));
  int* LC = malloc(sizeof(int) * NL * (size_t)(n_steps + 1) + 4);
  int* LV = malloc(sizeof(int) * NL * (size_t)(n_steps + 1) + 4);
  double* res = malloc(sizeof(double) * (NR + NL + 1));
  double *lam = calloc(6 * (size_t)N, sizeof(double)), *nxt = malloc(sizeof(double) * 6 * N);
  double* dLdy = malloc(sizeof(double) * N);
  G[0] = R[OR_DEFAULT_VM];
  G[1] = R[OR_DEFAULT_CA_NSR];
  memcpy(X, S0, sizeof(double) * 6 * N);
  memcpy(RY, ryr0, sizeof(int) * NR);
  memcpy(LC, lcc0, sizeof(int) * NL);
  memcpy(LV, lccv0, sizeof(int) * NL);
  memcpy(res, res0, sizeof(double) * (NR + NL));
  /* forward: x_{n+1} from x_n with the channel states of step n */
  for (n = 0; n < n_steps; ++n) {
    double* xn1 = X + 6 * (size_t)N * (n + 1);
    memcpy(xn1, X + 6 * (size_t)N * n, sizeof(double) * 6 * N);
    memcpy(RY + NR * (n + 1), RY + NR * n, sizeof(int) * NR);
    memcpy(LC + NL * (n + 1), LC + NL * n, sizeof(int) * NL);
    memcpy(LV + NL * (n + 1), LV + NL * n, sizeof(int) * NL);
    or_explicit_step(m, R, G, xn1, RY + NR * n, LC + NL * n, LV + NL * n);
    if (!I[OI_FLAG_NO_GATING])
      or_gating_philox(m, R, G[0], xn1, seed, n, RY + NR * (n + 1), LC + NL * (n + 1), LV + NL * (n + 1), res);
    if ((n + 1) % tick_every == 0)
      L += tick_loss(m, ns, W, pad, F0, target + (size_t)ns * ((n + 1) / tick_every - 1), xn1, NULL);
  }
  /* backward */
  for (k = 0; k < OR_N_ADJ; ++k) grad[k] = 0;
  for (n = n_steps; n >= 1; --n) {
    int j;
    if (n % tick_every == 0) {
      memset(dLdy, 0, sizeof(double) * N);
      tick_loss(m, ns, W, pad, F0, target + (size_t)ns * (n / tick_every - 1), X + 6 * (size_t)N * n, dLdy);
      for (j = 0; j < N; ++j) lam[S_DYE * N + j] += dLdy[j];
    }
    /* lam_{n-1} = lam_n + dt J(x_{n-1})^T lam_n */
    memcpy(nxt, lam, sizeof(double) * 6 * N);
    adj_step(m, R, G, X + 6 * (size_t)N * (n - 1), RY + NR * (n - 1), LC + NL * (n - 1), LV + NL * (n - 1), lam,
             nxt, grad);
    memcpy(lam, nxt, sizeof(double) * 6 * N);
  }
  if (lam0) memcpy(lam0, lam, sizeof(double) * 6 * N);
  free(X);
  free(RY);
  free(LC);
  free(LV);
  free(res);
  free(lam);
  free(nxt);
  free(dLdy);
  return L;
}

/* loss only (same forward), for finite differences */
double or_adjoint_loss(const or_mesh* m, const int* I, const double* R, const double* S0, const int* ryr0,
                       const int* lcc0, const int* lccv0, const double* res0, uint64_t seed, int64_t n_steps,
                       int tick_every, int ns, const double* W, const double* pad, const double* F0,
                       const double* target) {
  int N = m->N, NR = m->NR, NL = m->NL;
  int64_t n;
  double G[2], L = 0;
  double* S = malloc(sizeof(double) * 6 * N);
  int *ry = malloc(sizeof(int) * (NR + 1)), *lc = malloc(sizeof(int) * (NL + 1)), *lv = malloc(sizeof(int) * (NL + 1));
  double* res = malloc(sizeof(double) * (NR + NL + 1));
  G[0] = R[OR_DEFAULT_VM];
  G[1] = R[OR_DEFAULT_CA_NSR];
  memcpy(S, S0, sizeof(double) * 6 * N);
  memcpy(ry, ryr0, sizeof(int) * NR);
  memcpy(lc, lcc0, sizeof(int) * NL);
  memcpy(lv, lccv0, sizeof(int) * NL);
  memcpy(res, res0, sizeof(double) * (NR + NL));
  for (n = 0; n < n_steps; ++n) {
    or_explicit_step(m, R, G, S, ry, lc, lv);
    if (!I[OI_FLAG_NO_GATING]) or_gating_philox(m, R, G[0], S, seed, n, ry, lc, lv, res);
    if ((n + 1) % tick_every == 0)
      L += tick_loss(m, ns, W, pad, F0, target + (size_t)ns * ((n + 1) / tick_every - 1), S, NULL);
  }
  free(S);
  free(ry);
  free(lc);
  free(lv);
  free(res);
  return L;
}
