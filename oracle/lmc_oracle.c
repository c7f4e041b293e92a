/*
 * lmc_oracle.c - TEST ORACLE (see lmc_oracle.h): plain-C restatement of the
 * reference's lattice-MC hot path. Test infrastructure only; compiled with
 * -ffp-contract=off so its floating point follows the reference's operation
 * order exactly on both x86-64 and aarch64.
 *
 * Reference files restated here (paths inside the reference project):
 *   lmc/cfg/src/Config.cpp               GenerateFCC, ReassignLatticeVector, UpdateNeighbors,
 *                                        GetLatticePairCenter, GetLatticePairRotationMatrix,
 *                                        RotateLatticeVector, FindDistanceLabelBetweenLattice
 *   lmc/cfg/include/LatticeCluster.hpp   position / group comparators, LatticeCluster{MMM,MM2}
 *   lmc/cfg/include/ElementCluster.hpp   ElementCluster ordering
 *   lmc/pred/src/EnergyUtility.cpp       sorted lists, cluster mappings, one-hot encoding
 *   lmc/pred/src/VacancyMigrationPredictorQuartic.cpp, VacancyMigrationPredictorE0.cpp,
 *   lmc/pred/src/EnergyChangePredictorPairSite.cpp, EnergyPredictor.cpp
 *   lmc/mc/src/KineticMcAbstract.cpp, KineticMcFirstOmp.cpp, JumpEvent.cpp,
 *   lmc/mc/src/CanonicalMcAbstract.cpp, CanonicalMcOmp.cpp
 */
#include "lmc_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define EPS 1e-4 /* kEpsilon, VectorMatrix.hpp:65 */
static const double kLatticeConstant = 4.046;
static const double kCut1 = 3.5, kCut2 = 4.8, kCut3 = 5.3; /* Constants.hpp:8-11 */
static const double kBoltzmann = 8.617333262145e-5;
static const double kPrefactor = 1e13;
static const double kDeCounter[11] = {256, 1536, 768, 3072, 2048, 3072, 6144, 6144, 6144, 6144, 2048};
static const double kCensusCounter[11] = {256, 3072, 1536, 6144, 12288, 6144, 12288, 6144, 12288, 12288, 12288};

/* ------------------------------------------------------------------------- */
/* small helpers                                                              */
/* ------------------------------------------------------------------------- */
typedef int (*cmp_fn)(const void *a, const void *b, const void *ctx);

/* stable merge sort (std::sort order is irrelevant wherever ties occur here) */
static void msort_rec(char *base, char *tmp, size_t n, size_t sz, cmp_fn cmp, const void *ctx) {
  if (n < 2) return;
  size_t h = n / 2;
  msort_rec(base, tmp, h, sz, cmp, ctx);
  msort_rec(base + h * sz, tmp, n - h, sz, cmp, ctx);
  size_t i = 0, j = h, k = 0;
  while (i < h && j < n) {
    if (cmp(base + j * sz, base + i * sz, ctx) < 0) memcpy(tmp + (k++) * sz, base + (j++) * sz, sz);
    else memcpy(tmp + (k++) * sz, base + (i++) * sz, sz);
  }
  while (i < h) memcpy(tmp + (k++) * sz, base + (i++) * sz, sz);
  while (j < n) memcpy(tmp + (k++) * sz, base + (j++) * sz, sz);
  memcpy(base, tmp, n * sz);
}
static void msort(void *base, size_t n, size_t sz, cmp_fn cmp, const void *ctx) {
  if (n < 2) return;
  char *tmp = (char *)malloc(n * sz);
  msort_rec((char *)base, tmp, n, sz, cmp, ctx);
  free(tmp);
}
static int cmp_i64(const void *a, const void *b, const void *ctx) {
  (void)ctx;
  int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* ------------------------------------------------------------------------- */
/* lattice                                                                    */
/* ------------------------------------------------------------------------- */
struct orc_lattice {
  int n;
  int64_t N;
  double (*pos)[3];       /* relative positions by lattice id */
  int64_t (*nn)[42];      /* sorted 1NN(12) 2NN(6) 3NN(24) */
  int64_t *atom_lattice;  /* atom id (GenerateFCC order) -> lattice id */
  double L;               /* box edge (basis is diagonal) */
};

typedef struct {
  int64_t old_id;
  double p[3];
} gen_site;

/* Vector_d operator< (VectorMatrix.hpp:78-88) */
static int vec_less(const double *a, const double *b) {
  double dx = a[0] - b[0];
  if (dx < -EPS) return 1;
  if (dx > EPS) return 0;
  double dy = a[1] - b[1];
  if (dy < -EPS) return 1;
  if (dy > EPS) return 0;
  return a[2] < b[2] - EPS;
}
static int cmp_gen(const void *a, const void *b, const void *ctx) {
  (void)ctx;
  const gen_site *x = (const gen_site *)a, *y = (const gen_site *)b;
  if (vec_less(x->p, y->p)) return -1;
  if (vec_less(y->p, x->p)) return 1;
  return 0;
}

/* GetRelativeDistanceVectorLattice (Lattice.hpp:58-70) */
static void rel_dist(const double *a, const double *b, double *d) {
  for (int k = 0; k < 3; ++k) {
    double v = b[k] - a[k];
    while (v >= 0.5) v -= 1;
    while (v < -0.5) v += 1;
    d[k] = v;
  }
}

orc_lattice *orc_lattice_create(int n) {
  if (n < 4) return NULL;
  orc_lattice *lat = (orc_lattice *)calloc(1, sizeof(orc_lattice));
  lat->n = n;
  lat->N = 4LL * n * n * n;
  lat->L = kLatticeConstant * (double)n;
  gen_site *g = (gen_site *)malloc(sizeof(gen_site) * lat->N);
  /* GenerateFCC (Config.cpp:1060-1095) */
  int64_t count = 0;
  const double len = (double)n;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double x = (double)i, y = (double)j, z = (double)k;
        const double P[4][3] = {{x / len, y / len, z / len},
                                {(x + 0.5) / len, (y + 0.5) / len, z / len},
                                {(x + 0.5) / len, y / len, (z + 0.5) / len},
                                {x / len, (y + 0.5) / len, (z + 0.5) / len}};
        for (int q = 0; q < 4; ++q) {
          g[count].old_id = count;
          memcpy(g[count].p, P[q], sizeof(P[q]));
          ++count;
        }
      }
  /* ReassignLatticeVector (Config.cpp:466-552): new id = rank in position order */
  msort(g, (size_t)lat->N, sizeof(gen_site), cmp_gen, NULL);
  lat->pos = malloc(sizeof(double[3]) * lat->N);
  lat->atom_lattice = (int64_t *)malloc(sizeof(int64_t) * lat->N);
  for (int64_t id = 0; id < lat->N; ++id) {
    memcpy(lat->pos[id], g[id].p, sizeof(double) * 3);
    lat->atom_lattice[g[id].old_id] = id;
  }
  free(g);
  /* UpdateNeighbors (Config.cpp:955-1045): cell list, cutoffs 3.5/4.8/5.3 A */
  const int nc = (int)floor(lat->L / kCut3);
  int64_t *cell_of = (int64_t *)malloc(sizeof(int64_t) * lat->N);
  int64_t ncell = (int64_t)nc * nc * nc;
  int64_t *cnt = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  for (int64_t id = 0; id < lat->N; ++id) {
    int c[3];
    for (int q = 0; q < 3; ++q) c[q] = (int)floor((double)nc * lat->pos[id][q]);
    cell_of[id] = ((int64_t)c[0] * nc + c[1]) * nc + c[2];
    cnt[cell_of[id] + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) cnt[c + 1] += cnt[c];
  int64_t *members = (int64_t *)malloc(sizeof(int64_t) * lat->N);
  int64_t *fill = (int64_t *)calloc((size_t)ncell, sizeof(int64_t));
  for (int64_t id = 0; id < lat->N; ++id) members[cnt[cell_of[id]] + fill[cell_of[id]]++] = id;
  lat->nn = malloc(sizeof(int64_t[42]) * lat->N);
  const double c1 = kCut1 * kCut1, c2 = kCut2 * kCut2, c3 = kCut3 * kCut3;
  for (int64_t id = 0; id < lat->N; ++id) {
    int64_t l1[12], l2[6], l3[24];
    int n1 = 0, n2 = 0, n3 = 0;
    const int64_t cc = cell_of[id];
    const int ci = (int)(cc / ((int64_t)nc * nc)), cj = (int)((cc / nc) % nc), ck = (int)(cc % nc);
    for (int di = -1; di <= 1; ++di)
      for (int dj = -1; dj <= 1; ++dj)
        for (int dk = -1; dk <= 1; ++dk) {
          const int64_t nb = ((int64_t)((ci + di + nc) % nc) * nc + (cj + dj + nc) % nc) * nc + (ck + dk + nc) % nc;
          for (int64_t m = cnt[nb]; m < cnt[nb + 1]; ++m) {
            const int64_t o = members[m];
            if (o == id) continue;
            double d[3];
            rel_dist(lat->pos[id], lat->pos[o], d);
            double a[3] = {d[0] * lat->L, d[1] * lat->L, d[2] * lat->L};
            if (fabs(a[0]) > kCut3 || fabs(a[1]) > kCut3 || fabs(a[2]) > kCut3) continue;
            const double r2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
            int dup = 0;
            if (r2 < c1) {
              for (int q = 0; q < n1; ++q) dup |= l1[q] == o;
              if (!dup && n1 < 12) l1[n1++] = o;
            } else if (r2 < c2) {
              for (int q = 0; q < n2; ++q) dup |= l2[q] == o;
              if (!dup && n2 < 6) l2[n2++] = o;
            } else if (r2 < c3) {
              for (int q = 0; q < n3; ++q) dup |= l3[q] == o;
              if (!dup && n3 < 24) l3[n3++] = o;
            }
          }
        }
    msort(l1, (size_t)n1, 8, cmp_i64, NULL);
    msort(l2, (size_t)n2, 8, cmp_i64, NULL);
    msort(l3, (size_t)n3, 8, cmp_i64, NULL);
    memcpy(lat->nn[id], l1, 8 * 12);
    memcpy(lat->nn[id] + 12, l2, 8 * 6);
    memcpy(lat->nn[id] + 18, l3, 8 * 24);
  }
  free(cell_of);
  free(cnt);
  free(members);
  free(fill);
  return lat;
}

void orc_lattice_destroy(orc_lattice *lat) {
  if (!lat) return;
  free(lat->pos);
  free(lat->nn);
  free(lat->atom_lattice);
  free(lat);
}
int64_t orc_lattice_num_sites(const orc_lattice *lat) { return lat->N; }
void orc_lattice_neighbors(const orc_lattice *lat, int64_t id, int64_t *out42) { memcpy(out42, lat->nn[id], 8 * 42); }
void orc_lattice_position(const orc_lattice *lat, int64_t id, double *xyz) { memcpy(xyz, lat->pos[id], 24); }

int orc_distance_label(const orc_lattice *lat, int64_t a, int64_t b) {
  const int64_t *nn = lat->nn[a];
  for (int q = 0; q < 12; ++q)
    if (nn[q] == b) return 1;
  for (int q = 12; q < 18; ++q)
    if (nn[q] == b) return 2;
  for (int q = 18; q < 42; ++q)
    if (nn[q] == b) return 3;
  return -1;
}

/* ------------------------------------------------------------------------- */
/* pair frame and sorted lists                                                */
/* ------------------------------------------------------------------------- */
typedef struct {
  int64_t id;
  double p[3];
} site;

static void normalize(double *v) {
  const double f = 1.0 / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] *= f;
  v[1] *= f;
  v[2] *= f;
}

/* GetLatticePairCenter (Config.cpp:228-245) */
static void pair_center(const orc_lattice *lat, int64_t a, int64_t b, double *c) {
  for (int k = 0; k < 3; ++k) {
    double first = lat->pos[a][k];
    const double second = lat->pos[b][k];
    double distance = first - second;
    int period = (int)(distance / 0.5);
    while (period != 0) {
      first -= (double)period;
      distance = first - second;
      period = (int)(distance / 0.5);
    }
    c[k] = 0.5 * (first + second);
  }
}

/* GetLatticePairRotationMatrix (Config.cpp:247-264): R = transpose(rows d, v, d x v) */
static void pair_rotation(const orc_lattice *lat, int64_t a, int64_t b, double R[3][3]) {
  double d[3], v[3] = {0, 0, 0};
  rel_dist(lat->pos[a], lat->pos[b], d);
  for (int k = 0; k < 3; ++k) d[k] *= lat->L;
  normalize(d);
  for (int q = 0; q < 12; ++q) {
    double j[3];
    rel_dist(lat->pos[a], lat->pos[lat->nn[a][q]], j);
    for (int k = 0; k < 3; ++k) j[k] *= lat->L;
    normalize(j);
    const double dot = d[0] * j[0] + d[1] * j[1] + d[2] * j[2];
    if (fabs(dot) < EPS) {
      memcpy(v, j, sizeof(v));
      break;
    }
  }
  const double w[3] = {d[1] * v[2] - d[2] * v[1], d[2] * v[0] - d[0] * v[2], d[0] * v[1] - d[1] * v[0]};
  const double *rows[3] = {d, v, w};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[c][r] = rows[r][c];
}

/* Vector_d * Matrix_d (VectorMatrix.hpp) */
static void vec_mat(const double *x, double R[3][3], double *y) {
  for (int c = 0; c < 3; ++c) y[c] = x[0] * R[0][c] + x[1] * R[1][c] + x[2] * R[2][c];
}

/* RotateLatticeVector (Config.cpp:1047-1058) */
static void rotate_sites(site *s, int n, double R[3][3]) {
  const double half[3] = {0.5, 0.5, 0.5};
  double hr[3];
  vec_mat(half, R, hr);
  const double mv[3] = {0.5 - hr[0], 0.5 - hr[1], 0.5 - hr[2]};
  for (int i = 0; i < n; ++i) {
    double y[3];
    vec_mat(s[i].p, R, y);
    for (int k = 0; k < 3; ++k) {
      y[k] += mv[k];
      y[k] -= floor(y[k]);
    }
    memcpy(s[i].p, y, sizeof(y));
  }
}

static double inner_half(const double *p) {
  const double a = p[0] - 0.5, b = p[1] - 0.5, c = p[2] - 0.5;
  return a * a + b * b + c * c;
}

/* comparators of LatticeCluster.hpp:62-154, as 3-way compares */
static int pos_state(const site *l, const site *r) {
  const double dx = l->p[0] - r->p[0], dy = l->p[1] - r->p[1], dz = l->p[2] - r->p[2];
  if (dx < -EPS) return -1;
  if (dx > EPS) return 1;
  if (dy < -EPS) return -1;
  if (dy > EPS) return 1;
  if (dz < -EPS) return -1;
  if (dz > EPS) return 1;
  return 0;
}
static int pos_mmm(const site *l, const site *r) {
  const double dn = inner_half(l->p) - inner_half(r->p);
  if (dn < -EPS) return -1;
  if (dn > EPS) return 1;
  const double dxs = fabs(l->p[0] - 0.5) - fabs(r->p[0] - 0.5);
  if (dxs < -EPS) return -1;
  if (dxs > EPS) return 1;
  return pos_state(l, r);
}
static int pos_mm2(const site *l, const site *r) {
  const double dn = inner_half(l->p) - inner_half(r->p);
  if (dn < -EPS) return -1;
  if (dn > EPS) return 1;
  return pos_state(l, r);
}
static int group_mmm(const site *l, const site *r) {
  const double dn = inner_half(l->p) - inner_half(r->p);
  if (dn < -EPS) return -1;
  if (dn > EPS) return 1;
  const double dxs = fabs(l->p[0] - 0.5) - fabs(r->p[0] - 0.5);
  if (dxs < -EPS) return -1;
  if (dxs > EPS) return 1;
  return 0;
}
static int group_mm2(const site *l, const site *r) {
  const double dn = inner_half(l->p) - inner_half(r->p);
  if (dn < -EPS) return -1;
  if (dn > EPS) return 1;
  const double dx = l->p[0] - r->p[0];
  if (dx < -EPS) return -1;
  if (dx > EPS) return 1;
  return 0;
}
static int cmp_site_state(const void *a, const void *b, const void *c) { (void)c; return pos_state(a, b); }
static int cmp_site_mmm(const void *a, const void *b, const void *c) { (void)c; return pos_mmm(a, b); }
static int cmp_site_mm2(const void *a, const void *b, const void *c) { (void)c; return pos_mm2(a, b); }

/* GetNeighborsLatticeIdSetOf{Pair,Site} (Config.cpp:312-352) as a sorted unique list */
static int neighbor_set(const orc_lattice *lat, const int64_t *centers, int nc, int64_t *out) {
  int n = 0;
  for (int c = 0; c < nc; ++c) {
    const int64_t id = centers[c];
    int64_t cand[43];
    cand[0] = id;
    memcpy(cand + 1, lat->nn[id], 8 * 42);
    for (int q = 0; q < 43; ++q) {
      int dup = 0;
      for (int z = 0; z < n; ++z) dup |= out[z] == cand[q];
      if (!dup) out[n++] = cand[q];
    }
  }
  msort(out, (size_t)n, 8, cmp_i64, NULL);
  return n;
}

/* which: 0 state (all 60), 1 MMM, 2 MM2 (pair excluded) */
static int pair_sorted(const orc_lattice *lat, int64_t a, int64_t b, int which, site *out) {
  int64_t ids[128];
  const int64_t centers[2] = {a, b};
  const int nset = neighbor_set(lat, centers, 2, ids);
  double c[3];
  pair_center(lat, a, b, c);
  const double mv[3] = {0.5 - c[0], 0.5 - c[1], 0.5 - c[2]};
  int n = 0;
  for (int q = 0; q < nset; ++q) {
    site s;
    s.id = ids[q];
    for (int k = 0; k < 3; ++k) {
      double v = lat->pos[ids[q]][k];
      v += mv[k];
      v -= floor(v);
      s.p[k] = v;
    }
    if (which != 0 && (s.id == a || s.id == b)) continue;
    out[n++] = s;
  }
  double R[3][3];
  pair_rotation(lat, a, b, R);
  rotate_sites(out, n, R);
  msort(out, (size_t)n, sizeof(site), which == 0 ? cmp_site_state : (which == 1 ? cmp_site_mmm : cmp_site_mm2), NULL);
  return n;
}

/* GetSortedLatticeVectorStateOfSite (EnergyUtility.cpp:288-313): no rotation */
static int site_sorted(const orc_lattice *lat, int64_t a, site *out) {
  int64_t ids[64];
  const int nset = neighbor_set(lat, &a, 1, ids);
  const double mv[3] = {0.5 - lat->pos[a][0], 0.5 - lat->pos[a][1], 0.5 - lat->pos[a][2]};
  for (int q = 0; q < nset; ++q) {
    out[q].id = ids[q];
    for (int k = 0; k < 3; ++k) {
      double v = lat->pos[ids[q]][k];
      v += mv[k];
      v -= floor(v);
      out[q].p[k] = v;
    }
  }
  msort(out, (size_t)nset, sizeof(site), cmp_site_state, NULL);
  return nset;
}

int orc_pair_lists(const orc_lattice *lat, int64_t first, int64_t second, int64_t *state60, int64_t *mmm58,
                   int64_t *mm258) {
  site s[128];
  if (pair_sorted(lat, first, second, 0, s) != 60) return -1;
  if (state60)
    for (int k = 0; k < 60; ++k) state60[k] = s[k].id;
  if (pair_sorted(lat, first, second, 1, s) != 58) return -1;
  if (mmm58)
    for (int k = 0; k < 58; ++k) mmm58[k] = s[k].id;
  if (pair_sorted(lat, first, second, 2, s) != 58) return -1;
  if (mm258)
    for (int k = 0; k < 58; ++k) mm258[k] = s[k].id;
  return 0;
}

int orc_site_list(const orc_lattice *lat, int64_t a, int64_t *out43) {
  site s[64];
  if (site_sorted(lat, a, s) != 43) return -1;
  for (int k = 0; k < 43; ++k) out43[k] = s[k].id;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* cluster mappings                                                           */
/* ------------------------------------------------------------------------- */
typedef struct {
  int group;     /* label (state/site) or orbit index (MMM/MM2) */
  int size;
  int sym;       /* symmetric orbit flag (SIZE_MAX marker in the reference) */
  int idx[3];    /* indices into the sorted list */
} mcluster;

typedef struct {
  mcluster *c;
  int n, cap;
} mlist;

static void mpush(mlist *l, mcluster c) {
  if (l->n == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 256;
    l->c = (mcluster *)realloc(l->c, sizeof(mcluster) * (size_t)l->cap);
  }
  l->c[l->n++] = c;
}

/* GetLabel (EnergyUtility.cpp:345-379) on lattice ids */
static int label3(const orc_lattice *lat, int64_t a, int64_t b, int64_t c) {
  int l[3] = {orc_distance_label(lat, a, b), orc_distance_label(lat, b, c), orc_distance_label(lat, c, a)};
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j)
      if (l[j] < l[i]) {
        int t = l[i];
        l[i] = l[j];
        l[j] = t;
      }
  if (l[0] == 1 && l[1] == 1 && l[2] == 1) return 4;
  if (l[0] == 1 && l[1] == 1 && l[2] == 2) return 5;
  if (l[0] == 1 && l[1] == 1 && l[2] == 3) return 6;
  if (l[0] == 1 && l[1] == 2 && l[2] == 3) return 7;
  if (l[0] == 1 && l[1] == 3 && l[2] == 3) return 8;
  if (l[0] == 2 && l[1] == 3 && l[2] == 3) return 9;
  if (l[0] == 3 && l[1] == 3 && l[2] == 3) return 10;
  return -1;
}

/* GetClusterParametersMappingState{Pair,Site} (EnergyUtility.cpp:393-581):
 * clusters over the sorted list `s` that contain one of `centers`, grouped by
 * label 0..7 in the reference's loop order. */
static void state_mapping(const orc_lattice *lat, const site *s, int n, const int64_t *centers, int ncenters,
                          mlist *out) {
  mlist by[8] = {{0}};
  for (int i1 = 0; i1 < n; ++i1) {
    const int64_t id1 = s[i1].id;
    int c1 = 0;
    for (int q = 0; q < ncenters; ++q) c1 |= id1 == centers[q];
    if (c1) mpush(&by[0], (mcluster){0, 1, 0, {i1, 0, 0}});
    for (int i2 = 0; i2 < i1; ++i2) {
      const int64_t id2 = s[i2].id;
      int c2 = c1;
      for (int q = 0; q < ncenters; ++q) c2 |= id2 == centers[q];
      if (c2) {
        const int l = orc_distance_label(lat, id1, id2);
        if (l < 1) continue; /* `default: continue;` */
        mpush(&by[l], (mcluster){l, 2, 0, {i1, i2, 0}});
      }
      for (int i3 = 0; i3 < i2; ++i3) {
        const int64_t id3 = s[i3].id;
        int c3 = c2;
        for (int q = 0; q < ncenters; ++q) c3 |= id3 == centers[q];
        if (!c3) continue;
        const int l = label3(lat, id1, id2, id3);
        if (l >= 4 && l <= 7) mpush(&by[l], (mcluster){l, 3, 0, {i1, i2, i3}});
      }
    }
  }
  for (int l = 0; l < 8; ++l) {
    for (int q = 0; q < by[l].n; ++q) mpush(out, by[l].c[q]);
    free(by[l].c);
  }
}

typedef struct {
  const site *s;
  int mmm;
} env_ctx;

/* IsClusterSmallerSymmetrically{MMM,MM2} as a 3-way compare */
static int cmp_env_cluster(const void *a, const void *b, const void *ctx) {
  const mcluster *x = (const mcluster *)a, *y = (const mcluster *)b;
  const env_ctx *e = (const env_ctx *)ctx;
  for (int q = 0; q < x->size; ++q) {
    const site *l = &e->s[x->idx[q]], *r = &e->s[y->idx[q]];
    const int g = e->mmm ? group_mmm(l, r) : group_mm2(l, r);
    if (g) return g;
  }
  return 0;
}

/* GetAverageClusterParametersMapping{MMM,MM2} (EnergyUtility.cpp:106-259) */
static void env_mapping(const orc_lattice *lat, const site *s, int n, int mmm, mlist *out) {
  env_ctx ctx = {s, mmm};
  int orbit = 0;
  for (int label = 0; label <= 3; ++label) {
    mlist cl = {0};
    for (int i1 = 0; i1 < n; ++i1) {
      if (label == 0) {
        mpush(&cl, (mcluster){0, 1, 0, {i1, 0, 0}});
        continue;
      }
      for (int i2 = 0; i2 < i1; ++i2) {
        if (orc_distance_label(lat, s[i1].id, s[i2].id) != label) continue;
        /* LatticeCluster{MMM,MM2} constructor: sort the two lattices, then flag
         * clusters whose lattices fall in the same group */
        int a = i1, b = i2;
        const int pc = mmm ? pos_mmm(&s[a], &s[b]) : pos_mm2(&s[a], &s[b]);
        if (pc > 0) {
          int t = a;
          a = b;
          b = t;
        }
        const int g = mmm ? group_mmm(&s[a], &s[b]) : group_mm2(&s[a], &s[b]);
        mpush(&cl, (mcluster){0, 2, g == 0, {a, b, 0}});
      }
    }
    msort(cl.c, (size_t)cl.n, sizeof(mcluster), cmp_env_cluster, &ctx);
    for (int q = 0; q < cl.n; ++q) {
      if (q > 0 && cmp_env_cluster(&cl.c[q - 1], &cl.c[q], &ctx) != 0) ++orbit;
      mcluster c = cl.c[q];
      c.group = orbit;
      mpush(out, c);
    }
    if (cl.n > 0) ++orbit;
    free(cl.c);
  }
}

typedef struct {
  int ready;
  mlist state, site, mmm, mm2;
} mappings;

static void build_mappings(const orc_lattice *lat, mappings *m) {
  site s[128];
  memset(m, 0, sizeof(*m));
  const int64_t a = 0, b = lat->nn[0][0];
  const int64_t pc[2] = {a, b};
  int n = pair_sorted(lat, a, b, 0, s);
  state_mapping(lat, s, n, pc, 2, &m->state);
  n = site_sorted(lat, 0, s);
  state_mapping(lat, s, n, &a, 1, &m->site);
  n = pair_sorted(lat, a, b, 1, s);
  env_mapping(lat, s, n, 1, &m->mmm);
  n = pair_sorted(lat, a, b, 2, s);
  env_mapping(lat, s, n, 0, &m->mm2);
  m->ready = 1;
}

static void free_mappings(mappings *m) {
  free(m->state.c);
  free(m->site.c);
  free(m->mmm.c);
  free(m->mm2.c);
}

int orc_mapping(const orc_lattice *lat, int which, int32_t *out6, int cap) {
  mappings m;
  build_mappings(lat, &m);
  const mlist *l = which == 0 ? &m.state : which == 1 ? &m.site : which == 2 ? &m.mmm : &m.mm2;
  const int n = l->n;
  if (out6)
    for (int q = 0; q < n && q < cap; ++q) {
      out6[6 * q] = l->c[q].group;
      out6[6 * q + 1] = l->c[q].size;
      out6[6 * q + 2] = l->c[q].sym;
      for (int z = 0; z < 3; ++z) out6[6 * q + 3 + z] = l->c[q].idx[z];
    }
  free_mappings(&m);
  return n;
}

/* ------------------------------------------------------------------------- */
/* model                                                                     */
/* ------------------------------------------------------------------------- */
#define MAXE 6
typedef struct {
  int set;
  int k_mmm, k_mm2;
  double *mu_mmm, *sig_mmm, *mu_mm2, *sig_mm2, *u_mmm, *u_mm2, *th_d, *th_ks;
  double mu_d, sig_d, mu_ks, sig_ks;
} quartic_blk;
typedef struct {
  int set;
  int k;
  double *mu, *sig, *u, *th;
  double mu_e0, sig_e0;
} e0_blk;

struct orc_model {
  int E;                  /* alphabet size incl X */
  char names[MAXE][4];    /* string order */
  int x_code;
  int eh;                 /* one-hot alphabet size */
  int rank[MAXE];         /* one-hot rank per code or -1 */
  int num_theta;
  int key_size[512], key_label[512], key_codes[512][3];
  int16_t dense[8][MAXE][MAXE][MAXE]; /* (label, sorted codes) -> index or -1 */
  double *theta;
  quartic_blk q[MAXE];
  e0_blk e0[MAXE];
  /* mapping cache for the lattice the model was last used with */
  const orc_lattice *map_lat;
  mappings maps;
  /* multi-vacancy extension (orc_kmc_multi): a cluster with two vacancies or a
   * vacancy in a one-hot environment contributes nothing instead of an error */
  int x_zero;
};

static const char *kKnown[] = {"X", "Al", "Mg", "Zn", "Cu", "Sn"};

static int cmp_key(const int *sa, const int *la, const int *ca, const int *sb, const int *lb, const int *cb) {
  if (*sa != *sb) return *sa < *sb ? -1 : 1;
  if (*la != *lb) return *la < *lb ? -1 : 1;
  for (int q = 0; q < *sa; ++q)
    if (ca[q] != cb[q]) return ca[q] < cb[q] ? -1 : 1;
  return 0;
}

orc_model *orc_model_create(const char *const *names, int num_names) {
  orc_model *m = (orc_model *)calloc(1, sizeof(orc_model));
  char set[MAXE][4];
  int ns = 0;
  for (int i = 0; i < num_names + 1; ++i) {
    const char *nm = i < num_names ? names[i] : "X";
    int known = 0;
    for (int k = 0; k < 6; ++k) known |= strcmp(nm, kKnown[k]) == 0;
    if (!known) nm = "X"; /* Element(std::string) maps unknown names to X */
    int dup = 0;
    for (int k = 0; k < ns; ++k) dup |= strcmp(set[k], nm) == 0;
    if (!dup && ns < MAXE) {
      strncpy(set[ns], nm, 3);
      set[ns][3] = 0;
      ++ns;
    }
  }
  /* string order (std::set<Element>, Element::operator<) */
  for (int i = 0; i < ns; ++i)
    for (int j = i + 1; j < ns; ++j)
      if (strcmp(set[j], set[i]) < 0) {
        char t[4];
        memcpy(t, set[i], 4);
        memcpy(set[i], set[j], 4);
        memcpy(set[j], t, 4);
      }
  m->E = ns;
  for (int i = 0; i < ns; ++i) {
    memcpy(m->names[i], set[i], 4);
    if (strcmp(set[i], "X") == 0) m->x_code = i;
  }
  /* one-hot alphabet = the element set as given (unknown names -> X) */
  m->eh = 0;
  for (int c = 0; c < ns; ++c) {
    int in = 0;
    for (int i = 0; i < num_names; ++i) {
      int known = 0;
      for (int k = 0; k < 6; ++k) known |= strcmp(names[i], kKnown[k]) == 0;
      in |= strcmp(known ? names[i] : "X", set[c]) == 0;
    }
    m->rank[c] = in ? m->eh++ : -1;
  }
  /* InitializeClusterHashMap keys, std::map order */
  int n = 0;
  const int X = m->x_code;
  for (int c1 = 0; c1 < ns; ++c1) {
    m->key_size[n] = 1;
    m->key_label[n] = 0;
    m->key_codes[n][0] = c1;
    ++n;
  }
  for (int c1 = 0; c1 < ns; ++c1)
    for (int c2 = 0; c2 < ns; ++c2) {
      if (c2 == X) continue;
      for (int label = 1; label <= 3; ++label) {
        int k[3] = {c1 < c2 ? c1 : c2, c1 < c2 ? c2 : c1, 0};
        int dup = 0;
        for (int z = 0; z < n && !dup; ++z)
          dup = m->key_size[z] == 2 && m->key_label[z] == label && m->key_codes[z][0] == k[0] && m->key_codes[z][1] == k[1];
        if (!dup) {
          m->key_size[n] = 2;
          m->key_label[n] = label;
          memcpy(m->key_codes[n], k, sizeof(k));
          ++n;
        }
      }
      for (int c3 = 0; c3 < ns; ++c3) {
        if (c3 == X) continue;
        int k[3] = {c1, c2, c3};
        for (int i = 0; i < 3; ++i)
          for (int j = i + 1; j < 3; ++j)
            if (k[j] < k[i]) {
              int t = k[i];
              k[i] = k[j];
              k[j] = t;
            }
        for (int label = 4; label < 8; ++label) {
          int dup = 0;
          for (int z = 0; z < n && !dup; ++z)
            dup = m->key_size[z] == 3 && m->key_label[z] == label && m->key_codes[z][0] == k[0] &&
                  m->key_codes[z][1] == k[1] && m->key_codes[z][2] == k[2];
          if (!dup) {
            m->key_size[n] = 3;
            m->key_label[n] = label;
            memcpy(m->key_codes[n], k, sizeof(k));
            ++n;
          }
        }
      }
    }
  /* selection sort by (size, label, codes) */
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j)
      if (cmp_key(&m->key_size[j], &m->key_label[j], m->key_codes[j], &m->key_size[i], &m->key_label[i],
                  m->key_codes[i]) < 0) {
        int ts = m->key_size[i], tl = m->key_label[i], tc[3];
        memcpy(tc, m->key_codes[i], sizeof(tc));
        m->key_size[i] = m->key_size[j];
        m->key_label[i] = m->key_label[j];
        memcpy(m->key_codes[i], m->key_codes[j], sizeof(tc));
        m->key_size[j] = ts;
        m->key_label[j] = tl;
        memcpy(m->key_codes[j], tc, sizeof(tc));
      }
  m->num_theta = n;
  m->theta = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  memset(m->dense, 0xff, sizeof(m->dense));
  for (int z = 0; z < n; ++z) {
    const int *k = m->key_codes[z];
    m->dense[m->key_label[z]][k[0]][m->key_size[z] > 1 ? k[1] : 0][m->key_size[z] > 2 ? k[2] : 0] = (int16_t)z;
  }
  return m;
}

static void free_q(quartic_blk *q) {
  free(q->mu_mmm);
  free(q->sig_mmm);
  free(q->mu_mm2);
  free(q->sig_mm2);
  free(q->u_mmm);
  free(q->u_mm2);
  free(q->th_d);
  free(q->th_ks);
  memset(q, 0, sizeof(*q));
}
static void free_e(e0_blk *e) {
  free(e->mu);
  free(e->sig);
  free(e->u);
  free(e->th);
  memset(e, 0, sizeof(*e));
}

void orc_model_destroy(orc_model *m) {
  if (!m) return;
  for (int c = 0; c < MAXE; ++c) {
    free_q(&m->q[c]);
    free_e(&m->e0[c]);
  }
  if (m->maps.ready) free_mappings(&m->maps);
  free(m->theta);
  free(m);
}

int orc_model_num_species(const orc_model *m) { return m->E; }
void orc_model_set_vacancy_zero(orc_model *m, int on) { m->x_zero = on ? 1 : 0; }
int orc_model_num_theta(const orc_model *m) { return m->num_theta; }
int orc_model_code(const orc_model *m, const char *name) {
  for (int c = 0; c < m->E; ++c)
    if (strcmp(m->names[c], name) == 0) return c;
  return -1;
}

int orc_model_cluster_index(const orc_model *m, int label, int size, const int *codes) {
  /* ClusterIndexer::GetIndex: exact (label, sorted elements) key, -1 if absent */
  int k[3] = {0, 0, 0};
  for (int q = 0; q < size; ++q) k[q] = codes[q];
  for (int i = 0; i < size; ++i)
    for (int j = i + 1; j < size; ++j)
      if (k[j] < k[i]) {
        int t = k[i];
        k[i] = k[j];
        k[j] = t;
      }
  if (label < 0 || label > 7 || size != (label == 0 ? 1 : (label <= 3 ? 2 : 3))) return -1;
  return m->dense[label][k[0]][k[1]][k[2]];
}

static double *dup_arr(const double *p, size_t n) {
  double *d = (double *)malloc(sizeof(double) * (n ? n : 1));
  memcpy(d, p, sizeof(double) * n);
  return d;
}

static const mappings *maps_for(const orc_model *cm, const orc_lattice *lat) {
  orc_model *m = (orc_model *)cm;
  if (!m->maps.ready || m->map_lat != lat) {
    if (m->maps.ready) free_mappings(&m->maps);
    build_mappings(lat, &m->maps);
    m->map_lat = lat;
  }
  return &m->maps;
}

/* list_length of an orbit (GetOneHotParametersFromMap, EnergyUtility.cpp:755-759) */
static int block_len(const orc_model *m, const mcluster *c) {
  if (c->size == 1) return m->eh;
  return c->sym ? m->eh * (m->eh + 1) / 2 : m->eh * m->eh;
}

int orc_model_features(const orc_model *m, const orc_lattice *lat, int which) {
  const mappings *mp = maps_for(m, lat);
  const mlist *l = which == 2 ? &mp->mmm : &mp->mm2;
  int f = 0, last = -1;
  for (int q = 0; q < l->n; ++q)
    if (l->c[q].group != last) {
      f += block_len(m, &l->c[q]);
      last = l->c[q].group;
    }
  return f;
}

void orc_model_set_theta(orc_model *m, const double *theta, int n) {
  free(m->theta);
  m->theta = dup_arr(theta, (size_t)n);
}

void orc_model_set_quartic(orc_model *m, int code, int k_mmm, int f_mmm, int k_mm2, int f_mm2,
                           const double *mu_x_mmm, const double *sigma_x_mmm, const double *mu_x_mm2,
                           const double *sigma_x_mm2, const double *u_mmm, const double *u_mm2, const double *theta_d,
                           const double *theta_ks, double mu_d, double sigma_d, double mu_ks, double sigma_ks) {
  quartic_blk *q = &m->q[code];
  free_q(q);
  q->set = 1;
  q->k_mmm = k_mmm;
  q->k_mm2 = k_mm2;
  q->mu_mmm = dup_arr(mu_x_mmm, (size_t)f_mmm);
  q->sig_mmm = dup_arr(sigma_x_mmm, (size_t)f_mmm);
  q->mu_mm2 = dup_arr(mu_x_mm2, (size_t)f_mm2);
  q->sig_mm2 = dup_arr(sigma_x_mm2, (size_t)f_mm2);
  q->u_mmm = dup_arr(u_mmm, (size_t)k_mmm * f_mmm);
  q->u_mm2 = dup_arr(u_mm2, (size_t)k_mm2 * f_mm2);
  q->th_d = dup_arr(theta_d, (size_t)k_mmm);
  q->th_ks = dup_arr(theta_ks, (size_t)k_mm2);
  q->mu_d = mu_d;
  q->sig_d = sigma_d;
  q->mu_ks = mu_ks;
  q->sig_ks = sigma_ks;
}

void orc_model_set_e0(orc_model *m, int code, int k_mmm, int f_mmm, const double *mu_x_mmm,
                      const double *sigma_x_mmm, const double *u_mmm, const double *theta_e0, double mu_e0,
                      double sigma_e0) {
  e0_blk *e = &m->e0[code];
  free_e(e);
  e->set = 1;
  e->k = k_mmm;
  e->mu = dup_arr(mu_x_mmm, (size_t)f_mmm);
  e->sig = dup_arr(sigma_x_mmm, (size_t)f_mmm);
  e->u = dup_arr(u_mmm, (size_t)k_mmm * f_mmm);
  e->th = dup_arr(theta_e0, (size_t)k_mmm);
  e->mu_e0 = mu_e0;
  e->sig_e0 = sigma_e0;
}

/* ------------------------------------------------------------------------- */
/* predictors                                                                 */
/* ------------------------------------------------------------------------- */

/* one-hot numerators of one mapping over an element vector (codes), as
 * GetOneHotParametersFromMap (EnergyUtility.cpp:743-796) before the division */
static int onehot_counts(const orc_model *m, const mlist *l, const int *codes, int32_t *out, int *fsize) {
  int off = 0, last = -1, blk = 0;
  for (int q = 0; q < l->n; ++q) {
    const mcluster *c = &l->c[q];
    if (c->group != last) {
      off += blk;
      blk = block_len(m, c);
      for (int z = 0; z < blk; ++z) out[off + z] = 0;
      last = c->group;
    }
    int r[2], skip = 0;
    for (int z = 0; z < c->size; ++z) {
      r[z] = m->rank[codes[c->idx[z]]];
      if (r[z] < 0) {
        if (!m->x_zero) return -3; /* one_hot_encode_hashmap.at() throws */
        skip = 1;                  /* a vacancy: zero one-hot vector */
      }
    }
    if (skip) continue;
    int t;
    if (c->size == 1) t = r[0];
    else if (!c->sym) t = r[0] * m->eh + r[1];
    else {
      /* sorted strings joined by '-': rank order equals string order */
      const int lo = r[0] < r[1] ? r[0] : r[1], hi = r[0] < r[1] ? r[1] : r[0];
      t = lo * m->eh - lo * (lo - 1) / 2 + (hi - lo);
    }
    out[off + t] += 1;
  }
  *fsize = off + blk;
  return 0;
}

static void orbit_sizes(const mlist *l, const orc_model *m, int *sizes) {
  int off = 0, last = -1, blk = 0, start = 0;
  for (int q = 0; q <= l->n; ++q) {
    if (q == l->n || l->c[q].group != last) {
      if (last >= 0)
        for (int z = 0; z < blk; ++z) sizes[off + z] = q - start;
      if (q == l->n) break;
      off += blk;
      blk = block_len(m, &l->c[q]);
      last = l->c[q].group;
      start = q;
    }
  }
}

/* The reference's per-(site, slot) tables site_bond_cluster_{state,mmm,mm2}_flat_
 * (VacancyMigrationPredictorQuartic.cpp:64-100), computed for one pair. */
typedef struct {
  int32_t st[60], mmm[58], mm2f[58], mm2b[58];
} pair_ids;

static int make_pair_ids(const orc_lattice *lat, int64_t a, int64_t b, pair_ids *p) {
  site s[128];
  if (pair_sorted(lat, a, b, 0, s) != 60) return -1;
  for (int k = 0; k < 60; ++k) p->st[k] = (int32_t)s[k].id;
  if (pair_sorted(lat, a, b, 1, s) != 58) return -1;
  for (int k = 0; k < 58; ++k) p->mmm[k] = (int32_t)s[k].id;
  if (pair_sorted(lat, a, b, 2, s) != 58) return -1;
  for (int k = 0; k < 58; ++k) p->mm2f[k] = (int32_t)s[k].id;
  if (pair_sorted(lat, b, a, 2, s) != 58) return -1;
  for (int k = 0; k < 58; ++k) p->mm2b[k] = (int32_t)s[k].id;
  return 0;
}

/* GetDe (VacancyMigrationPredictorQuartic.cpp:112-166): counts and dE */
static int de_from_ids(const orc_model *m, const mappings *mp, const int8_t *sp, int64_t a, int64_t b,
                       const int32_t *ids, int32_t *cs, int32_t *ce, double *de) {
  const int mig = sp[b];
  int32_t s0[512], e0[512];
  for (int z = 0; z < m->num_theta; ++z) s0[z] = e0[z] = 0;
  for (int q = 0; q < mp->state.n; ++q) {
    const mcluster *c = &mp->state.c[q];
    int st[3], en[3];
    for (int z = 0; z < c->size; ++z) {
      const int64_t id = ids[c->idx[z]];
      st[z] = sp[id];
      en[z] = id == a ? mig : (id == b ? m->x_code : sp[id]);
    }
    const int is = orc_model_cluster_index(m, c->group, c->size, st);
    const int ie = orc_model_cluster_index(m, c->group, c->size, en);
    if ((is < 0 || ie < 0) && !m->x_zero) return -2;
    if (is >= 0) s0[is]++; /* x_zero: a cluster outside the indexer counts nothing */
    if (ie >= 0) e0[ie]++;
  }
  double acc = 0.0;
  for (int z = 0; z < m->num_theta; ++z) {
    const double enc = ((double)e0[z] - (double)s0[z]) / kDeCounter[m->key_label[z]];
    const double p = m->theta[z] * enc;
    acc = acc + p;
  }
  if (cs) memcpy(cs, s0, sizeof(int32_t) * m->num_theta);
  if (ce) memcpy(ce, e0, sizeof(int32_t) * m->num_theta);
  *de = acc;
  return 0;
}

/* standardise, U x, dot theta (VacancyMigrationPredictorQuartic.cpp:203-214,234-245) */
static double linear_form(const double *x, int f, const double *mu, const double *sig, const double *u, int k,
                          const double *th, double sig_y, double mu_y) {
  double z[4096];
  for (int j = 0; j < f; ++j) z[j] = x[j] - mu[j];
  for (int j = 0; j < f; ++j) z[j] = z[j] / sig[j];
  double out = 0.0;
  for (int r = 0; r < k; ++r) {
    double s = 0.0;
    for (int j = 0; j < f; ++j) {
      const double p = u[(size_t)r * f + j] * z[j];
      s = s + p;
    }
    const double p = s * th[r];
    out = out + p;
  }
  out *= sig_y;
  out += mu_y;
  return out;
}

/* one-hot features of a 58-site list (counts and/or averaged values) */
static int env_from_ids(const orc_model *m, const mlist *l, const int8_t *sp, const int32_t *ids, double *x,
                        int32_t *counts, int *f) {
  int codes[64];
  for (int k = 0; k < 58; ++k) codes[k] = sp[ids[k]];
  int32_t tmp[4096];
  int32_t *cnt = counts ? counts : tmp;
  const int rc = onehot_counts(m, l, codes, cnt, f);
  if (rc) return rc;
  if (x) {
    int sz[4096];
    orbit_sizes(l, m, sz);
    for (int j = 0; j < *f; ++j) x[j] = (double)cnt[j] / (double)sz[j];
  }
  return 0;
}

/* GetBarrierAndDiffFromLatticeIdPair of the Quartic (kind 0, out = Ea, dE, D, Ks)
 * or E0 (kind 1, out = Ea, dE, e0) predictor from precomputed id lists */
static int barrier_from_ids(const orc_model *m, const mappings *mp, const int8_t *sp, int64_t a, int64_t b,
                            const pair_ids *p, int kind, double *out) {
  const int mig = sp[b];
  if (kind == 0 && !m->q[mig].set) return -4;
  if (kind == 1 && !m->e0[mig].set) return -4;
  double dE;
  int rc, fm, f2;
  if ((rc = de_from_ids(m, mp, sp, a, b, p->st, NULL, NULL, &dE))) return rc;
  double xm[4096];
  if ((rc = env_from_ids(m, &mp->mmm, sp, p->mmm, xm, NULL, &fm))) return rc;
  if (kind == 1) {
    const e0_blk *e = &m->e0[mig];
    const double e0 = exp(linear_form(xm, fm, e->mu, e->sig, e->u, e->k, e->th, e->sig_e0, e->mu_e0));
    const double h = e0 + dE / 2;
    out[0] = h > 0.0 ? h : 0.0; /* std::max(0.0, e0 + dE / 2) */
    out[1] = dE;
    out[2] = e0;
    return 0;
  }
  const quartic_blk *q = &m->q[mig];
  double xf[4096], xb[4096];
  if ((rc = env_from_ids(m, &mp->mm2, sp, p->mm2f, xf, NULL, &f2))) return rc;
  if ((rc = env_from_ids(m, &mp->mm2, sp, p->mm2b, xb, NULL, &f2))) return rc;
  const double D = exp(linear_form(xm, fm, q->mu_mmm, q->sig_mmm, q->u_mmm, q->k_mmm, q->th_d, q->sig_d, q->mu_d));
  for (int j = 0; j < f2; ++j) xf[j] = xf[j] + xb[j];
  const double Ks =
      exp(linear_form(xf, f2, q->mu_mm2, q->sig_mm2, q->u_mm2, q->k_mm2, q->th_ks, q->sig_ks, q->mu_ks));
  /* closed form, VacancyMigrationPredictorQuartic.cpp:269-274 */
  const double bb = 4 * dE / (D * D * D);
  const double aa = Ks / (4 * D * D);
  const double c = (9 * bb * bb - 16 * aa * aa * D * D) / (32 * aa);
  const double delta = sqrt(fabs(9 * bb * bb - 32 * aa * c));
  const double Ea = (3 * bb + delta) * (3 * bb + delta) * (3 * bb * bb - 16 * aa * c + bb * delta) / pow(aa, 3) / 2048;
  out[0] = Ea;
  out[1] = dE;
  out[2] = D;
  out[3] = Ks;
  return 0;
}

int orc_encode(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t first, int64_t second,
               int32_t *state_start, int32_t *state_end, int32_t *mmm, int32_t *mm2f, int32_t *mm2b) {
  if (orc_distance_label(lat, first, second) != 1) return -1;
  const mappings *mp = maps_for(m, lat);
  pair_ids p;
  double de;
  int f, rc;
  if ((rc = make_pair_ids(lat, first, second, &p))) return rc;
  if ((rc = de_from_ids(m, mp, sp, first, second, p.st, state_start, state_end, &de))) return rc;
  if (mmm && (rc = env_from_ids(m, &mp->mmm, sp, p.mmm, NULL, mmm, &f))) return rc;
  if (mm2f && (rc = env_from_ids(m, &mp->mm2, sp, p.mm2f, NULL, mm2f, &f))) return rc;
  if (mm2b && (rc = env_from_ids(m, &mp->mm2, sp, p.mm2b, NULL, mm2b, &f))) return rc;
  return 0;
}

int orc_quartic(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t first, int64_t second,
                double *out4) {
  if (orc_distance_label(lat, first, second) != 1) return -1;
  pair_ids p;
  if (make_pair_ids(lat, first, second, &p)) return -1;
  return barrier_from_ids(m, maps_for(m, lat), sp, first, second, &p, 0, out4);
}

int orc_e0(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t first, int64_t second,
           double *out3) {
  if (orc_distance_label(lat, first, second) != 1) return -1;
  pair_ids p;
  if (make_pair_ids(lat, first, second, &p)) return -1;
  return barrier_from_ids(m, maps_for(m, lat), sp, first, second, &p, 1, out3);
}

/* GetDeHelper (EnergyChangePredictorPairSite.cpp:83-94) */
static double de_helper(const orc_model *m, const int32_t *s0, const int32_t *e0) {
  double acc = 0.0;
  for (int z = 0; z < m->num_theta; ++z) {
    const double enc = ((double)e0[z] - (double)s0[z]) / kDeCounter[m->key_label[z]];
    const double p = m->theta[z] * enc;
    acc = acc + p;
  }
  return acc;
}

/* GetDeFromLatticeIdSite (EnergyChangePredictorPairSite.cpp:154-192) */
static int site_de(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t a, int newc, double *de) {
  if (sp[a] == newc) {
    *de = 0.0;
    return 0;
  }
  const mappings *mp = maps_for(m, lat);
  site s[64];
  site_sorted(lat, a, s);
  int32_t s0[512], e0[512];
  for (int z = 0; z < m->num_theta; ++z) s0[z] = e0[z] = 0;
  for (int q = 0; q < mp->site.n; ++q) {
    const mcluster *c = &mp->site.c[q];
    int st[3], en[3];
    for (int z = 0; z < c->size; ++z) {
      const int64_t id = s[c->idx[z]].id;
      st[z] = sp[id];
      en[z] = id == a ? newc : sp[id];
    }
    const int is = orc_model_cluster_index(m, c->group, c->size, st);
    const int ie = orc_model_cluster_index(m, c->group, c->size, en);
    if (is < 0 || ie < 0) return -2;
    s0[is]++;
    e0[ie]++;
  }
  *de = de_helper(m, s0, e0);
  return 0;
}

/* EnergyChangePredictorPairSite::GetDeFromLatticeIdSite (EnergyChangePredictorPairSite.cpp:154-192). */
int orc_site_de(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t site, int new_code, double *de) {
  return site_de(m, lat, sp, site, new_code, de);
}

int orc_pair_site_de(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t a, int64_t b,
                     double *de) {
  const int ca = sp[a], cb = sp[b];
  if (ca == cb) {
    *de = 0.0;
    return 0;
  }
  int coupled = a == b;
  for (int q = 0; q < 42; ++q) coupled |= lat->nn[a][q] == b;
  if (!coupled) {
    double d1, d2;
    int rc;
    if ((rc = site_de(m, lat, sp, a, cb, &d1))) return rc;
    if ((rc = site_de(m, lat, sp, b, ca, &d2))) return rc;
    *de = d1 + d2;
    return 0;
  }
  /* coupled: GetClusterParametersMappingStatePairOf (EnergyUtility.cpp:582-663)
   * over the union set, clusters containing a or b */
  int64_t ids[128];
  const int64_t centers[2] = {a, b};
  const int n = neighbor_set(lat, centers, 2, ids);
  site s[128];
  for (int q = 0; q < n; ++q) s[q].id = ids[q];
  mlist l = {0};
  state_mapping(lat, s, n, centers, 2, &l);
  int32_t s0[512], e0[512];
  for (int z = 0; z < m->num_theta; ++z) s0[z] = e0[z] = 0;
  int rc = 0;
  for (int q = 0; q < l.n && !rc; ++q) {
    const mcluster *c = &l.c[q];
    int st[3], en[3];
    for (int z = 0; z < c->size; ++z) {
      const int64_t id = s[c->idx[z]].id;
      st[z] = sp[id];
      en[z] = id == a ? cb : (id == b ? ca : sp[id]);
    }
    const int is = orc_model_cluster_index(m, c->group, c->size, st);
    const int ie = orc_model_cluster_index(m, c->group, c->size, en);
    if (is < 0 || ie < 0) rc = -2;
    else {
      s0[is]++;
      e0[ie]++;
    }
  }
  free(l.c);
  if (rc) return rc;
  *de = de_helper(m, s0, e0);
  return 0;
}

int orc_energy(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t *counts, double *energy) {
  int64_t c[512];
  for (int z = 0; z < m->num_theta; ++z) c[z] = 0;
  for (int64_t l1 = 0; l1 < lat->N; ++l1) {
    const int e1 = sp[l1];
    const int64_t *n1 = lat->nn[l1];
    int k[3] = {e1, 0, 0};
    int idx = orc_model_cluster_index(m, 0, 1, k);
    if (idx < 0 && !m->x_zero) return -2;
    if (idx >= 0) c[idx]++; /* x_zero: unindexed clusters count nothing */
    for (int a = 0; a < 12; ++a) {
      const int64_t l2 = n1[a];
      k[1] = sp[l2];
      if ((idx = orc_model_cluster_index(m, 1, 2, k)) < 0 && !m->x_zero) return -2;
      if (idx >= 0) c[idx]++; /* x_zero: unindexed clusters count nothing */
      for (int b = 0; b < 12; ++b) {
        const int64_t l3 = lat->nn[l2][b];
        int label = -1;
        for (int q = 0; q < 12 && label < 0; ++q)
          if (n1[q] == l3) label = 4;
        for (int q = 12; q < 18 && label < 0; ++q)
          if (n1[q] == l3) label = 5;
        for (int q = 18; q < 42 && label < 0; ++q)
          if (n1[q] == l3) label = 6;
        if (label < 0) continue;
        k[2] = sp[l3];
        if ((idx = orc_model_cluster_index(m, label, 3, k)) < 0 && !m->x_zero) return -2;
        if (idx >= 0) c[idx]++; /* x_zero: unindexed clusters count nothing */
      }
      for (int b = 12; b < 18; ++b) {
        const int64_t l3 = lat->nn[l2][b];
        int in3 = 0;
        for (int q = 18; q < 42; ++q) in3 |= n1[q] == l3;
        if (!in3) continue;
        k[2] = sp[l3];
        if ((idx = orc_model_cluster_index(m, 7, 3, k)) < 0 && !m->x_zero) return -2;
        if (idx >= 0) c[idx]++; /* x_zero: unindexed clusters count nothing */
      }
    }
    for (int a = 12; a < 18; ++a) {
      int kk[3] = {e1, sp[n1[a]], 0};
      if ((idx = orc_model_cluster_index(m, 2, 2, kk)) < 0 && !m->x_zero) return -2;
      if (idx >= 0) c[idx]++; /* x_zero: unindexed clusters count nothing */
    }
    for (int a = 18; a < 42; ++a) {
      int kk[3] = {e1, sp[n1[a]], 0};
      if ((idx = orc_model_cluster_index(m, 3, 2, kk)) < 0 && !m->x_zero) return -2;
      if (idx >= 0) c[idx]++; /* x_zero: unindexed clusters count nothing */
    }
  }
  double acc = 0.0;
  for (int z = 0; z < m->num_theta; ++z) {
    const double enc = (double)c[z] / kCensusCounter[m->key_label[z]];
    const double p = m->theta[z] * enc;
    acc = acc + p;
  }
  if (counts) memcpy(counts, c, sizeof(int64_t) * m->num_theta);
  if (energy) *energy = acc;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* solute clusters (ansys::SoluteCluster, SoluteCluster.cpp:277-410)          */
/* ------------------------------------------------------------------------- */
/* EnergyPredictor::GetEncodeOfCluster + GetEnergyOfCluster (EnergyPredictor.cpp:97-184): the census
 * restricted to S = the listed sites and their 1-3NN neighbours (every site of a counted cluster in
 * S), species taken from sp, or the solvent everywhere except at the listed sites (mode 1), or the
 * solvent everywhere (mode 2). */
int orc_cluster_energy(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int solvent, int mode,
                       const int64_t *sites, int64_t count, double *energy) {
  unsigned char *in_s = (unsigned char *)calloc((size_t)lat->N, 1);
  unsigned char *in_l = (unsigned char *)calloc((size_t)lat->N, 1);
  int64_t *list = (int64_t *)malloc(sizeof(int64_t) * (size_t)(count * 43 + 1));
  if (!in_s || !in_l || !list) {
    free(in_s);
    free(in_l);
    free(list);
    return -5;
  }
  int64_t ns = 0;
  for (int64_t i = 0; i < count; ++i) {
    const int64_t a = sites[i];
    in_l[a] = 1;
    if (!in_s[a]) in_s[a] = 1, list[ns++] = a;
    for (int q = 0; q < 42; ++q) {
      const int64_t b = lat->nn[a][q];
      if (!in_s[b]) in_s[b] = 1, list[ns++] = b;
    }
  }
#define ORC_SP(x) (mode == 0 ? sp[x] : (mode == 1 && in_l[x] ? sp[x] : solvent))
  int64_t c[512];
  int rc = 0;
  for (int z = 0; z < m->num_theta; ++z) c[z] = 0;
  for (int64_t t = 0; t < ns && rc == 0; ++t) {
    const int64_t l1 = list[t];
    const int64_t *n1 = lat->nn[l1];
    int k[3] = {ORC_SP(l1), 0, 0};
    int idx = orc_model_cluster_index(m, 0, 1, k);
    if (idx < 0 && !m->x_zero) { rc = -2; break; }
    if (idx >= 0) c[idx]++;
    for (int a = 0; a < 12 && rc == 0; ++a) {
      const int64_t l2 = n1[a];
      if (!in_s[l2]) continue;
      k[1] = ORC_SP(l2);
      if ((idx = orc_model_cluster_index(m, 1, 2, k)) < 0 && !m->x_zero) { rc = -2; break; }
      if (idx >= 0) c[idx]++;
      for (int b = 0; b < 12; ++b) {
        const int64_t l3 = lat->nn[l2][b];
        if (!in_s[l3]) continue;
        int label = -1;
        for (int q = 0; q < 12 && label < 0; ++q)
          if (n1[q] == l3) label = 4;
        for (int q = 12; q < 18 && label < 0; ++q)
          if (n1[q] == l3) label = 5;
        for (int q = 18; q < 42 && label < 0; ++q)
          if (n1[q] == l3) label = 6;
        if (label < 0) continue;
        k[2] = ORC_SP(l3);
        if ((idx = orc_model_cluster_index(m, label, 3, k)) < 0 && !m->x_zero) { rc = -2; break; }
        if (idx >= 0) c[idx]++;
      }
      for (int b = 12; b < 18 && rc == 0; ++b) {
        const int64_t l3 = lat->nn[l2][b];
        if (!in_s[l3]) continue;
        int in3 = 0;
        for (int q = 18; q < 42; ++q) in3 |= n1[q] == l3;
        if (!in3) continue;
        k[2] = ORC_SP(l3);
        if ((idx = orc_model_cluster_index(m, 7, 3, k)) < 0 && !m->x_zero) { rc = -2; break; }
        if (idx >= 0) c[idx]++;
      }
    }
    for (int a = 12; a < 42 && rc == 0; ++a) {
      if (!in_s[n1[a]]) continue;
      int kk[3] = {ORC_SP(l1), ORC_SP(n1[a]), 0};
      if ((idx = orc_model_cluster_index(m, a < 18 ? 2 : 3, 2, kk)) < 0 && !m->x_zero) { rc = -2; break; }
      if (idx >= 0) c[idx]++;
    }
  }
#undef ORC_SP
  free(in_s);
  free(in_l);
  free(list);
  if (rc) return rc;
  double acc = 0.0;
  for (int z = 0; z < m->num_theta; ++z) {
    const double enc = (double)c[z] / kCensusCounter[m->key_label[z]];
    const double p = m->theta[z] * enc;
    acc = acc + p;
  }
  *energy = acc;
  return 0;
}

static int cmp_id(const void *a, const void *b) {
  const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return x < y ? -1 : x > y;
}
typedef struct {
  int64_t *ids;
  int64_t size;
} orc_cl;
static int cmp_cluster(const void *a, const void *b) {
  const orc_cl *x = (const orc_cl *)a, *y = (const orc_cl *)b;
  if (x->size != y->size) return x->size > y->size ? -1 : 1;
  return x->ids[0] < y->ids[0] ? -1 : x->ids[0] > y->ids[0];
}

/* SoluteCluster::FindAtomListOfClusters (SoluteCluster.cpp:277-373): connected components of the
 * non-solvent sites under 1NN bonds (breadth-first, as FindAtomListOfClustersBFSHelper), components
 * smaller than `smallest` dropped; a component of more than `bond` sites gains every site of its 1NN
 * shell with more than `bond` 1NN bonds to it. Clusters sorted by size, larger first (ties: smaller
 * first site id first; the reference leaves their order to std::sort over hash-set order), members
 * sorted by id. offsets (K + 1) and members (capacity `cap`) receive the CSR lists; returns K or a
 * negative error. */
int64_t orc_solute_clusters(const orc_lattice *lat, const int8_t *sp, int solvent, int64_t smallest, int64_t bond,
                            int64_t *offsets, int64_t *members, int64_t cap) {
  const int64_t N = lat->N;
  unsigned char *seen = (unsigned char *)calloc((size_t)N, 1);
  int64_t *queue = (int64_t *)malloc(sizeof(int64_t) * (size_t)N);
  orc_cl *cl = (orc_cl *)malloc(sizeof(orc_cl) * (size_t)(N + 1));
  int64_t *mark = (int64_t *)malloc(sizeof(int64_t) * (size_t)N);
  if (!seen || !queue || !cl || !mark) {
    free(seen), free(queue), free(cl), free(mark);
    return -5;
  }
  for (int64_t i = 0; i < N; ++i) mark[i] = -1;
  int64_t K = 0;
  for (int64_t s0 = 0; s0 < N; ++s0) {
    if (sp[s0] == solvent || seen[s0]) continue;
    int64_t head = 0, tail = 0;
    queue[tail++] = s0;
    seen[s0] = 1;
    while (head < tail) {
      const int64_t a = queue[head++];
      for (int q = 0; q < 12; ++q) {
        const int64_t b = lat->nn[a][q];
        if (sp[b] != solvent && !seen[b]) seen[b] = 1, queue[tail++] = b;
      }
    }
    if (tail < smallest) continue;
    /* the component, then its qualifying solvent shell */
    int64_t cap_k = tail * 13;
    int64_t *ids = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap_k);
    int64_t size = 0;
    for (int64_t i = 0; i < tail; ++i) ids[size++] = queue[i], mark[queue[i]] = K;
    if (tail > bond) {
      for (int64_t i = 0; i < tail; ++i) {
        for (int q = 0; q < 12; ++q) {
          const int64_t c = lat->nn[queue[i]][q];
          if (mark[c] == K) continue; /* already a member */
          int64_t bonds = 0;
          for (int r = 0; r < 12; ++r) {
            const int64_t d = lat->nn[c][r];
            bonds += mark[d] == K && sp[d] != solvent;
          }
          if (bonds > bond) {
            ids[size++] = c;
            mark[c] = K;
          }
        }
      }
    }
    for (int64_t i = 0; i < size; ++i)
      if (sp[ids[i]] == solvent) mark[ids[i]] = -1; /* solvent sites may join several clusters */
    qsort(ids, (size_t)size, sizeof(int64_t), cmp_id);
    cl[K].ids = ids;
    cl[K].size = size;
    ++K;
  }
  qsort(cl, (size_t)K, sizeof(orc_cl), cmp_cluster);
  int64_t off = 0, rc = K;
  offsets[0] = 0;
  for (int64_t k = 0; k < K; ++k) {
    if (off + cl[k].size > cap) rc = -1;
    for (int64_t i = 0; i < cl[k].size && off + i < cap; ++i) members[off + i] = cl[k].ids[i];
    off += cl[k].size;
    offsets[k + 1] = off;
    free(cl[k].ids);
  }
  free(seen), free(queue), free(cl), free(mark);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* random numbers                                                             */
/* ------------------------------------------------------------------------- */
void orc_mt_seed(orc_mt *g, uint64_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 312; ++i) g->mt[i] = 6364136223846793005ULL * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
  g->idx = 312;
}

uint64_t orc_mt_next(orc_mt *g) {
  if (g->idx >= 312) {
    for (int k = 0; k < 312; ++k) {
      const uint64_t x = (g->mt[k] & 0xFFFFFFFF80000000ULL) | (g->mt[(k + 1) % 312] & 0x7FFFFFFFULL);
      g->mt[k] = g->mt[(k + 156) % 312] ^ (x >> 1) ^ ((x & 1ULL) ? 0xB5026F5AA96619E9ULL : 0ULL);
    }
    g->idx = 0;
  }
  uint64_t y = g->mt[g->idx++];
  y ^= (y >> 29) & 0x5555555555555555ULL;
  y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
  y ^= (y << 37) & 0xFFF7EEE000000000ULL;
  y ^= y >> 43;
  return y;
}

double orc_mt_uniform(orc_mt *g) {
  const double u = (double)orc_mt_next(g) * 5.421010862427522170e-20; /* 2^-64 */
  return u >= 1.0 ? nextafter(1.0, 0.0) : u;
}

uint64_t orc_mt_below(orc_mt *g, uint64_t range) {
  /* Lemire's multiply-and-reject (ACM TOMACS 29(1), 2019) on 64-bit draws */
  uint64_t x = orc_mt_next(g);
  unsigned __int128 prod = (unsigned __int128)x * range;
  uint64_t low = (uint64_t)prod;
  if (low < range) {
    const uint64_t threshold = (0 - range) % range;
    while (low < threshold) {
      x = orc_mt_next(g);
      prod = (unsigned __int128)x * range;
      low = (uint64_t)prod;
    }
  }
  return (uint64_t)(prod >> 64);
}

/* ------------------------------------------------------------------------- */
/* drivers                                                                    */
/* ------------------------------------------------------------------------- */
typedef struct {
  uint8_t key[176];
  double ea, de;
  int used;
} memo_entry;

typedef struct {
  int64_t key; /* site * 12 + slot, -1 = empty */
  pair_ids ids;
} ids_entry;

static uint64_t fnv(const uint8_t *k, int n) {
  uint64_t h = 1469598103934665603ULL;
  for (int i = 0; i < n; ++i) h = (h ^ k[i]) * 1099511628211ULL;
  return h;
}

/* TimeTemperatureInterpolator::GetTemperature (TimeTemperatureInterpolator.cpp:44-65):
 * first point with time >= t (std::lower_bound), clamped at both ends, linear between. */
static double interp_temperature(const double *tt, const double *tv, int len, double t) {
  int lo = 0;
  while (lo < len && tt[lo] < t) ++lo;
  if (lo == len) return tv[len - 1];
  if (lo == 0 && t <= tt[0]) return tv[0];
  const double ux = tt[lo], uy = tv[lo], lx = tt[lo - 1], ly = tv[lo - 1];
  const double dy = uy - ly, dx = ux - lx;
  return ly + ((t - lx) / dx) * dy;
}

/* RateCorrector::GetTimeCorrectionFactor (RateCorrector.hpp:17-24). */
static double time_correction(double cvac, double csol, double T) {
  const double cv = 1.64 * exp(-(0.66 / kBoltzmann / T - 0.7));
  return cvac / cv / (1 - 13 * csol);
}

int orc_kmc(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps, int kind,
            int memo, double *trace8, double *events36) {
  return orc_kmc_ex(m, lat, sp, T, seed, steps, kind, memo, trace8, events36, NULL, NULL, 0, 0, 0, NULL);
}

/* Config::GetSolventElement (Config.cpp:411-422): the most frequent element. */
static int solvent_code(const orc_model *m, const orc_lattice *lat, const int8_t *sp) {
  int64_t count[MAXE] = {0};
  for (int64_t i = 0; i < lat->N; ++i) ++count[sp[i]];
  int best = 0;
  for (int c = 1; c < m->E; ++c)
    if (count[c] > count[best]) best = c;
  return best;
}

int orc_kmc_ex(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps,
               int kind, int memo, double *trace8, double *events36, const double *tt_time, const double *tt_temp,
               int tt_len, int rate_corrector, int early_stop, int64_t *steps_done) {
  const int solvent = early_stop ? solvent_code(m, lat, sp) : -1;
  if (steps_done) *steps_done = 0;
  orc_mt g;
  orc_mt_seed(&g, seed);
  const mappings *mp = maps_for(m, lat);
  double beta = 1.0 / kBoltzmann / T;
  /* RateCorrector(config.GetVacancyConcentration(), config.GetSoluteConcentration(Element("Al")))
   * (KineticMcAbstract.cpp:35; Config.cpp:373-391) */
  double cvac = 0.0, csol = 0.0;
  if (rate_corrector) {
    int al = -1;
    for (int c = 0; c < m->E; ++c)
      if (strcmp(m->names[c], "Al") == 0) al = c;
    int64_t nx = 0, ns = 0;
    for (int64_t i = 0; i < lat->N; ++i) {
      if (sp[i] == m->x_code) ++nx;
      else if (sp[i] != al) ++ns;
    }
    cvac = (double)nx / (double)lat->N;
    csol = (double)ns / (double)lat->N;
  }
  /* GetVacancyLatticeId: first X in atom order (Config.cpp:298-310) */
  int64_t vac = -1;
  for (int64_t at = 0; at < lat->N && vac < 0; ++at)
    if (sp[lat->atom_lattice[at]] == m->x_code) vac = lat->atom_lattice[at];
  if (vac < 0) return -1;
  /* lazily filled per-(site, slot) id lists, as the predictor constructor's tables */
  const size_t icap = (size_t)1 << 14;
  ids_entry *itab = (ids_entry *)malloc(icap * sizeof(ids_entry));
  for (size_t q = 0; q < icap; ++q) itab[q].key = -1;
  size_t iused = 0;
  /* barrier memo keyed by the exact species signature (the LRU's role) */
  const size_t cap = (size_t)1 << 17;
  memo_entry *tab = memo ? (memo_entry *)calloc(cap, sizeof(memo_entry)) : NULL;
  size_t used = 0;
  double time = 0.0, energy = 0.0;
  int rc = 0;
  for (int64_t st = 0; st < steps && !rc; ++st) {
    /* KineticMcFirstAbstract::UpdateTemperature (KineticMcAbstract.cpp:45-50) */
    if (tt_len > 0) {
      T = interp_temperature(tt_time, tt_temp, tt_len, time);
      beta = 1.0 / kBoltzmann / T;
    }
    double ea[12], de[12], k[12];
    const int64_t *nb = lat->nn[vac];
    double total = 0.0;
    for (int i = 0; i < 12 && !rc; ++i) {
      const int64_t j = nb[i];
      const int64_t ikey = vac * 12 + i;
      size_t h = (size_t)((uint64_t)ikey * 0x9E3779B97F4A7C15ULL >> 50) & (icap - 1);
      while (itab[h].key != -1 && itab[h].key != ikey) h = (h + 1) & (icap - 1);
      if (itab[h].key == -1) {
        if (iused > icap / 2) {
          for (size_t q = 0; q < icap; ++q) itab[q].key = -1;
          iused = 0;
          h = (size_t)((uint64_t)ikey * 0x9E3779B97F4A7C15ULL >> 50) & (icap - 1);
        }
        if ((rc = make_pair_ids(lat, vac, j, &itab[h].ids))) break;
        itab[h].key = ikey;
        ++iused;
      }
      const pair_ids *p = &itab[h].ids;
      memo_entry *slot = NULL;
      uint8_t key[176];
      if (memo) {
        for (int q = 0; q < 60; ++q) key[q] = (uint8_t)sp[p->st[q]];
        for (int q = 0; q < 58; ++q) key[60 + q] = (uint8_t)sp[p->mmm[q]];
        for (int q = 0; q < 58; ++q) key[118 + q] = (uint8_t)sp[p->mm2f[q]];
        size_t hh = (size_t)(fnv(key, 176) & (cap - 1));
        while (tab[hh].used && memcmp(tab[hh].key, key, 176) != 0) hh = (hh + 1) & (cap - 1);
        slot = &tab[hh];
        if (slot->used) {
          ea[i] = slot->ea;
          de[i] = slot->de;
        }
      }
      if (!slot || !slot->used) {
        double o[4];
        if ((rc = barrier_from_ids(m, mp, sp, vac, j, p, kind, o))) break;
        ea[i] = o[0];
        de[i] = o[1];
        if (slot) {
          if (used > cap / 2) {
            memset(tab, 0, cap * sizeof(memo_entry));
            used = 0;
            slot = &tab[(size_t)(fnv(key, 176) & (cap - 1))];
          }
          memcpy(slot->key, key, 176);
          slot->ea = ea[i];
          slot->de = de[i];
          slot->used = 1;
          ++used;
        }
      }
      k[i] = exp(-ea[i] * beta); /* JumpEvent forward rate (JumpEvent.cpp:6-13) */
      total += k[i];
    }
    if (rc) break;
    double cum[12], cp = 0.0;
    for (int i = 0; i < 12; ++i) {
      cp += k[i] / total;
      cum[i] = cp;
    }
    const double u1 = orc_mt_uniform(&g);
    /* CalculateTime() * GetTimeCorrectionFactor() (KineticMcAbstract.cpp:52-57,146) */
    const double dt = -log(u1) / total / kPrefactor * (rate_corrector ? time_correction(cvac, csol, T) : 1.0);
    const double u2 = orc_mt_uniform(&g);
    int sel = 11;
    for (int i = 0; i < 12; ++i)
      if (!(cum[i] < u2)) {
        sel = i;
        break;
      }
    const int64_t j = nb[sel];
    if (events36)
      for (int i = 0; i < 12; ++i) {
        events36[st * 36 + 3 * i] = (double)nb[i];
        events36[st * 36 + 3 * i + 1] = ea[i];
        events36[st * 36 + 3 * i + 2] = de[i];
      }
    time += dt;
    energy += de[sel];
    if (trace8) {
      double *t = trace8 + st * 8;
      t[0] = (double)vac;
      t[1] = (double)j;
      t[2] = sel;
      t[3] = ea[sel];
      t[4] = de[sel];
      t[5] = total;
      t[6] = time;
      t[7] = energy;
    }
    /* KineticMcFirstAbstract::IsEscaped (KineticMcAbstract.cpp:192-223): checked on the
     * configuration before the jump; the step completes, then the run ends */
    int escaped = 0;
    if (early_stop) {
      escaped = 1;
      for (int q = 0; q < 42; ++q)
        if (sp[nb[q]] != solvent) escaped = 0;
    }
    sp[vac] = sp[j];
    sp[j] = (int8_t)m->x_code;
    vac = j;
    if (steps_done) *steps_done = st + 1;
    if (escaped) break;
  }
  free(tab);
  free(itab);
  return rc;
}

/* KineticMcFirstOmp's step with the 12 jump barriers evaluated by `threads` OpenMP threads, as
 * KineticMcFirstOmp.cpp:52-82 parallelises that loop; the id lists of every (site, jump) are built
 * before the steps, as the predictor's constructor builds its tables. Rates, sums, draws, selection
 * and move are orc_kmc_ex's (no rate corrector, schedule or early stop), so the trajectory is
 * orc_kmc's. *loop_s receives the wall time of the step loop alone. Returns 0, or -1. */
int orc_kmc_threads(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps,
                    int kind, int threads, double *trace8, double *loop_s) {
  orc_mt g;
  orc_mt_seed(&g, seed);
  const mappings *mp = maps_for(m, lat); /* built before any parallel region */
  const double beta = 1.0 / kBoltzmann / T;
  int64_t vac = -1;
  for (int64_t at = 0; at < lat->N && vac < 0; ++at)
    if (sp[lat->atom_lattice[at]] == m->x_code) vac = lat->atom_lattice[at];
  if (vac < 0 || threads < 1) return -1;
  pair_ids *ids = (pair_ids *)malloc(sizeof(pair_ids) * (size_t)lat->N * 12);
  if (!ids) return -1;
  int failed = 0;
#pragma omp parallel for num_threads(threads) schedule(static) reduction(| : failed)
  for (int64_t q = 0; q < lat->N * 12; ++q)
    if (make_pair_ids(lat, q / 12, lat->nn[q / 12][q % 12], &ids[q])) failed |= 1;
  if (failed) {
    free(ids);
    return -1;
  }
  double time = 0.0, energy = 0.0;
  int rc = 0;
  const double t0 = omp_get_wtime();
  for (int64_t st = 0; st < steps; ++st) {
    double ea[12], de[12], k[12];
    const int64_t *nb = lat->nn[vac];
    int bad = 0;
#pragma omp parallel for num_threads(threads) schedule(static, 1) reduction(| : bad)
    for (int i = 0; i < 12; ++i) {
      double o[4];
      if (barrier_from_ids(m, mp, sp, vac, nb[i], &ids[vac * 12 + i], kind, o)) {
        bad |= 1;
      } else {
        ea[i] = o[0];
        de[i] = o[1];
      }
    }
    if (bad) {
      rc = -1;
      break;
    }
    double total = 0.0;
    for (int i = 0; i < 12; ++i) {
      k[i] = exp(-ea[i] * beta); /* JumpEvent forward rate (JumpEvent.cpp:6-13) */
      total += k[i];
    }
    double cum[12], cp = 0.0;
    for (int i = 0; i < 12; ++i) {
      cp += k[i] / total;
      cum[i] = cp;
    }
    const double u1 = orc_mt_uniform(&g);
    const double dt = -log(u1) / total / kPrefactor;
    const double u2 = orc_mt_uniform(&g);
    int sel = 11;
    for (int i = 0; i < 12; ++i)
      if (!(cum[i] < u2)) {
        sel = i;
        break;
      }
    const int64_t j = nb[sel];
    time += dt;
    energy += de[sel];
    if (trace8) {
      double *t = trace8 + st * 8;
      t[0] = (double)vac;
      t[1] = (double)j;
      t[2] = sel;
      t[3] = ea[sel];
      t[4] = de[sel];
      t[5] = total;
      t[6] = time;
      t[7] = energy;
    }
    sp[vac] = sp[j];
    sp[j] = (int8_t)m->x_code;
    vac = j;
  }
  if (loop_s) *loop_s = omp_get_wtime() - t0;
  free(ids);
  return rc;
}

int64_t orc_cmc(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t attempts,
                int batch, double *energy_io, double *energy_trace, int64_t cap, int64_t *accepted) {
  orc_mt g;
  orc_mt_seed(&g, seed);
  (void)maps_for(m, lat); /* build the mappings before any parallel region */
  const double beta = 1.0 / kBoltzmann / T;
  const uint64_t N = (uint64_t)lat->N;
  uint8_t *mark = (uint8_t *)calloc(N, 1);
  int64_t *marked = (int64_t *)malloc(sizeof(int64_t) * (size_t)batch * 86);
  int64_t (*pairs)[2] = malloc(sizeof(int64_t[2]) * (size_t)batch);
  double *des = (double *)malloc(sizeof(double) * (size_t)batch);
  double energy = *energy_io;
  int64_t done = 0, acc = 0;
  while (done < attempts) {
    /* BuildEventVector (CanonicalMcOmp.cpp:40-79) */
    int nb = 0;
    int64_t nm = 0;
    for (int i = 0; i < batch; ++i) {
      int ct = 0;
      int64_t l1, l2;
      for (;;) {
        do {
          l1 = (int64_t)orc_mt_below(&g, N);
          l2 = (int64_t)orc_mt_below(&g, N);
        } while (sp[l1] == sp[l2]);
        ++ct;
        if (ct == 50) break;
        if (!mark[l1] && !mark[l2]) break;
      }
      if (ct == 50) break;
      const int64_t ends[2] = {l1, l2};
      for (int e = 0; e < 2; ++e) {
        if (!mark[ends[e]]) {
          mark[ends[e]] = 1;
          marked[nm++] = ends[e];
        }
        for (int q = 0; q < 42; ++q) {
          const int64_t id = lat->nn[ends[e]][q];
          if (!mark[id]) {
            mark[id] = 1;
            marked[nm++] = id;
          }
        }
      }
      pairs[nb][0] = l1;
      pairs[nb][1] = l2;
      ++nb;
    }
    /* the batch's dE on the unchanged lattice, one pair per OpenMP thread
     * (CanonicalMcOmp.cpp:75-78) */
    int failed = 0;
#pragma omp parallel for schedule(static) reduction(| : failed)
    for (int i = 0; i < nb; ++i) failed |= orc_pair_site_de(m, lat, sp, pairs[i][0], pairs[i][1], &des[i]) != 0;
    if (failed) {
      done = -1;
      break;
    }
    /* sequential Metropolis (CanonicalMcAbstract.cpp:86-101) */
    for (int i = 0; i < nb; ++i) {
      if (energy_trace && done < cap) energy_trace[done] = energy;
      const double dE = des[i];
      int ok = dE < 0;
      if (!ok) {
        const double p = exp(-dE * beta);
        ok = orc_mt_uniform(&g) < p;
      }
      if (ok) {
        const int8_t t = sp[pairs[i][0]];
        sp[pairs[i][0]] = sp[pairs[i][1]];
        sp[pairs[i][1]] = t;
        energy += dE;
        ++acc;
      }
      ++done;
    }
    for (int64_t q = 0; q < nm; ++q) mark[marked[q]] = 0;
    if (nb == 0) break;
  }
  free(mark);
  free(marked);
  free(pairs);
  free(des);
  *energy_io = energy;
  if (accepted) *accepted = acc;
  return done;
}

/* ------------------------------------------------------------------------- */
/* Multi-vacancy KMC (the project's extension, restated from its definition:  */
/* the reference tracks one vacancy)                                          */
/* ------------------------------------------------------------------------- */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies, key bumped by the
 * Weyl constants after each round. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c1 = (uint32_t)p1;
    c3 = (uint32_t)p0;
    c0 = n0;
    c2 = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* The production KMC draws of lattice r at step s: -log(u1), u1 in (0, 1], and
 * u2 in [0, 1), 53 bits each, from Philox(counter = (s, r, "KMC"), key = seed). */
static void philox_step_draws(uint64_t seed, uint64_t step, uint32_t r, double *nlog_u1, double *u2) {
  const uint32_t ctr[4] = {(uint32_t)step, (uint32_t)(step >> 32), r, 0x4b4d43u};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t x[4];
  orc_philox4x32_10(ctr, key, x);
  const uint64_t a = (((uint64_t)x[0] << 32) | x[1]) >> 11, b = (((uint64_t)x[2] << 32) | x[3]) >> 11;
  *nlog_u1 = -log((double)(a + 1) * 1.1102230246251565404e-16);
  *u2 = (double)b * 1.1102230246251565404e-16;
}

/* inclusive scan of n (16 or 32) values in log2(n) doubling steps:
 * v[i] <- v[i] + v[i - o] for i >= o, o = 1, 2, 4, ... */
static void doubling_scan(double *v, int n) {
  double t[32];
  for (int o = 1; o < n; o <<= 1) {
    memcpy(t, v, sizeof(double) * n);
    for (int i = o; i < n; ++i) v[i] = t[i] + t[i - o];
  }
}

int orc_kmc_multi(orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, uint32_t replica,
                  uint64_t step0, int64_t steps, int kind, int64_t *vac, int nv, double *time_io, double *energy_io,
                  double *trace9) {
  if (nv < 1 || nv > 256) return -1;
  const mappings *mp = maps_for(m, lat);
  const double beta = 1.0 / kBoltzmann / T;
  double *cum = (double *)malloc(sizeof(double) * 16 * nv);
  double *ea = (double *)malloc(sizeof(double) * 12 * nv), *de = (double *)malloc(sizeof(double) * 12 * nv);
  double *kk = (double *)malloc(sizeof(double) * 12 * nv), *incl = (double *)malloc(sizeof(double) * nv);
  double time = *time_io, energy = *energy_io;
  int rc = 0;
  const int saved = m->x_zero;
  m->x_zero = 1;
  for (int64_t s = 0; s < steps && !rc; ++s) {
    /* every slot: its 12 events in id order, rates and their 16-wide scan */
    for (int v = 0; v < nv && !rc; ++v) {
      const int64_t *nb = lat->nn[vac[v]];
      double *c = cum + 16 * v;
      for (int j = 0; j < 12; ++j) {
        ea[12 * v + j] = de[12 * v + j] = kk[12 * v + j] = 0.0;
        if (sp[nb[j]] == m->x_code) continue; /* onto a vacancy: rate 0 */
        pair_ids p;
        double o[4];
        if ((rc = make_pair_ids(lat, vac[v], nb[j], &p))) break;
        if ((rc = barrier_from_ids(m, mp, sp, vac[v], nb[j], &p, kind, o))) break;
        ea[12 * v + j] = o[0];
        de[12 * v + j] = o[1];
        kk[12 * v + j] = exp(-o[0] * beta);
      }
      for (int j = 0; j < 16; ++j) c[j] = j < 12 ? kk[12 * v + j] : 0.0;
      doubling_scan(c, 16);
    }
    if (rc) break;
    /* prefix of the slot totals, 32 slots at a time */
    double run = 0.0;
    for (int c0 = 0; c0 < nv; c0 += 32) {
      double w[32];
      for (int i = 0; i < 32; ++i) w[i] = c0 + i < nv ? cum[16 * (c0 + i) + 11] : 0.0;
      doubling_scan(w, 32);
      for (int i = 0; i < 32 && c0 + i < nv; ++i) incl[c0 + i] = run + w[i];
      run = run + w[31];
    }
    const double total = run;
    double nlog_u1, u2;
    philox_step_draws(seed, step0 + (uint64_t)s, replica, &nlog_u1, &u2);
    const double xs = u2 * total;
    int vsel = -1, vlast = -1;
    for (int v = 0; v < nv; ++v) {
      if (!(cum[16 * v + 11] > 0.0)) continue;
      vlast = v;
      if (vsel < 0 && incl[v] >= xs) vsel = v;
    }
    if (vsel < 0) vsel = vlast;
    if (vsel < 0 || !(total > 0.0) || !isfinite(total)) {
      rc = -5;
      break;
    }
    const double y = xs - (vsel > 0 ? incl[vsel - 1] : 0.0);
    int sel = -1, jlast = -1;
    for (int j = 0; j < 12; ++j) {
      if (!(kk[12 * vsel + j] > 0.0)) continue;
      jlast = j;
      if (sel < 0 && cum[16 * vsel + j] >= y) sel = j;
    }
    if (sel < 0) sel = jlast;
    const int64_t from = vac[vsel], to = lat->nn[from][sel];
    time += nlog_u1 / (total * kPrefactor);
    energy += de[12 * vsel + sel];
    sp[from] = sp[to];
    sp[to] = (int8_t)m->x_code;
    vac[vsel] = to;
    if (trace9) {
      double *t = trace9 + 9 * s;
      t[0] = vsel;
      t[1] = (double)from;
      t[2] = (double)to;
      t[3] = sel;
      t[4] = ea[12 * vsel + sel];
      t[5] = de[12 * vsel + sel];
      t[6] = total;
      t[7] = time;
      t[8] = energy;
    }
  }
  m->x_zero = saved;
  *time_io = time;
  *energy_io = energy;
  free(cum);
  free(ea);
  free(de);
  free(kk);
  free(incl);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Second-order "chain" KMC (KineticMcChainOmpi.cpp:56-152, KineticMcAbstract.cpp:140-190,260-263) */
/* ------------------------------------------------------------------------- */

int orc_kmc_chain(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps,
                  int kind, int rng, uint32_t replica, double *trace8) {
  orc_mt g;
  orc_mt_seed(&g, seed);
  const mappings *mp = maps_for(m, lat);
  const double beta = 1.0 / kBoltzmann / T;
  int64_t vac = -1;
  for (int64_t at = 0; at < lat->N && vac < 0; ++at)
    if (sp[lat->atom_lattice[at]] == m->x_code) vac = lat->atom_lattice[at];
  if (vac < 0) return -1;
  int64_t prev = lat->nn[vac][0]; /* previous_j_lattice_id_: first 1NN of the initial vacancy */
  double time = 0.0, energy = 0.0;
  for (int64_t st = 0; st < steps; ++st) {
    const int64_t k = vac;
    const int64_t *nbk = lat->nn[k];
    double total_i[12], barrier_ki[12], de_ki[12], rate_ki[12], back_ki[12];
    /* BuildEventList: per neighbour i, the 12 jumps i -> l after the jump k -> i */
    for (int r = 0; r < 12; ++r) {
      const int64_t i = nbk[r];
      sp[k] = sp[i];
      sp[i] = (int8_t)m->x_code;
      double tot = 0.0, ea_ik = 0.0, de_ik = 0.0;
      for (int q = 0; q < 12; ++q) {
        const int64_t l = lat->nn[i][q];
        pair_ids p;
        double o[4];
        int rc;
        if ((rc = make_pair_ids(lat, i, l, &p)) || (rc = barrier_from_ids(m, mp, sp, i, l, &p, kind, o))) {
          sp[i] = sp[k];
          sp[k] = (int8_t)m->x_code;
          return rc;
        }
        tot += exp(-o[0] * beta);
        if (l == k) {
          ea_ik = o[0];
          de_ik = o[1];
        }
      }
      sp[i] = sp[k];
      sp[k] = (int8_t)m->x_code;
      /* event_k_i_ = event_i_l.GetReverseJumpEvent() (JumpEvent.cpp:54-57) */
      barrier_ki[r] = ea_ik - de_ik;
      de_ki[r] = -de_ik;
      rate_ki[r] = exp(-barrier_ki[r] * beta);                 /* forward rate */
      back_ki[r] = exp((de_ki[r] - barrier_ki[r]) * beta);      /* GetBackwardRate */
      total_i[r] = tot;
    }
    double total_k = 0.0;
    for (int r = 0; r < 12; ++r) total_k += rate_ki[r];
    /* CalculateTime: sums over the 12 events in rank order */
    const double t_1 = 1 / total_k / kPrefactor;
    double beta_bar_k = 0, beta_k = 0, gamma_bar_k_j = 0, gamma_k_j = 0, beta_k_j = 0, alpha_k_j = 0, ts_num = 0,
           ts_j_num = 0, bb[12], bk[12];
    int is_prev[12];
    for (int r = 0; r < 12; ++r) {
      const double p_ki = rate_ki[r] / total_k;
      const double p_ik = back_ki[r] / total_i[r];
      bb[r] = p_ki * p_ik;
      bk[r] = p_ki * (1 - p_ik);
      is_prev[r] = nbk[r] == prev;
      const double t_i = 1 / total_i[r] / kPrefactor;
      beta_bar_k += bb[r];
      beta_k += bk[r];
      gamma_bar_k_j += is_prev[r] ? 0.0 : bb[r];
      gamma_k_j += is_prev[r] ? 0.0 : bk[r];
      beta_k_j += is_prev[r] ? bk[r] : 0.0;
      alpha_k_j += is_prev[r] ? p_ki : 0.0;
      ts_num += (t_1 + t_i) * bb[r];
      ts_j_num += is_prev[r] ? 0.0 : (t_1 + t_i) * bb[r];
    }
    const double ts = ts_num / beta_bar_k;
    const double ts_j = ts_j_num / gamma_bar_k_j;
    const double one_over = 1 / (1 - alpha_k_j);
    const double t_2 = one_over * (gamma_k_j * t_1 + gamma_bar_k_j * (ts_j + t_1 + beta_bar_k / beta_k * ts));
    double cum[12], c = 0.0;
    for (int r = 0; r < 12; ++r) {
      const double pr = is_prev[r] ? one_over * (gamma_bar_k_j / beta_k) * beta_k_j
                                   : one_over * (1 + gamma_bar_k_j / beta_k) * bk[r];
      c += pr;
      cum[r] = c;
    }
    /* SelectEvent: one draw (the time is deterministic) */
    double u;
    if (rng == 0) {
      u = orc_mt_uniform(&g);
    } else {
      double nl;
      philox_step_draws(seed, (uint64_t)st, replica, &nl, &u);
    }
    int sel = 11;
    for (int r = 0; r < 12; ++r)
      if (!(cum[r] < u)) {
        sel = r;
        break;
      }
    const int64_t j = nbk[sel];
    time += t_2;
    energy += de_ki[sel];
    if (trace8) {
      double *t = trace8 + st * 8;
      t[0] = (double)k;
      t[1] = (double)j;
      t[2] = sel;
      t[3] = barrier_ki[sel];
      t[4] = de_ki[sel];
      t[5] = total_k;
      t[6] = time;
      t[7] = energy;
    }
    sp[k] = sp[j];
    sp[j] = (int8_t)m->x_code;
    prev = k;
    vac = j;
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Simulated annealing (SimulatedAnnealing.cpp:78-185) on a given lattice      */
/* ------------------------------------------------------------------------- */

int orc_sa(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T0, uint64_t seed, uint64_t maximum_steps,
           int64_t steps, double energy0, double *trace7, double *state4) {
  const double eps = 1e-4; /* kEpsilon, VectorMatrix.hpp:65 */
  orc_mt g;
  orc_mt_seed(&g, seed);
  const uint64_t N = (uint64_t)lat->N;
#define SA_FRAC(r) ((uint64_t)((double)maximum_steps * (r)) > 1 ? (uint64_t)((double)maximum_steps * (r)) : 1)
  const uint64_t reheat_trigger = SA_FRAC(0.05), reheat_cooldown = SA_FRAC(0.10), window_size = SA_FRAC(0.001);
#undef SA_FRAC
  double T = T0, beta = 1.0 / kBoltzmann / T0, energy = energy0, lowest = energy0, recent_best = energy0;
  uint64_t last_improvement = 0, last_reheat = 0, st = 0;
  unsigned window_trials = 0, window_accepts = 0, reheats_done = 0;
  for (int64_t s = 0; s < steps; ++s, ++st) {
    if (energy < lowest - eps) lowest = energy; /* Dump */
    int64_t l1, l2;
    do {
      l1 = (int64_t)orc_mt_below(&g, N);
      l2 = (int64_t)orc_mt_below(&g, N);
    } while (sp[l1] == sp[l2]);
    double dE;
    int rc = orc_pair_site_de(m, lat, sp, l1, l2, &dE);
    if (rc) return rc;
    const double e_before = energy, t_before = T;
    int accepted = dE < 0;
    if (!accepted) accepted = orc_mt_uniform(&g) < exp(-dE * beta);
    if (accepted) {
      const int8_t v = sp[l1];
      sp[l1] = sp[l2];
      sp[l2] = v;
      energy += dE;
    }
    /* UpdateTemperature (SimulatedAnnealing.cpp:99-137) */
    ++window_trials;
    if (accepted) {
      ++window_accepts;
      if (energy < recent_best - eps) {
        recent_best = energy;
        last_improvement = st;
      }
    }
    if (window_trials >= window_size) {
      const double acc = (double)window_accepts / (double)window_trials;
      if (acc > 0.50) T *= 0.99;
      window_trials = 0;
      window_accepts = 0;
    }
    const double acc_est = window_trials > 0u ? (double)window_accepts / (double)window_trials : 1.0;
    if (reheats_done < 5 && st - last_improvement >= reheat_trigger && st - last_reheat >= reheat_cooldown &&
        acc_est < 0.05) {
      T *= 1.10;
      last_improvement = st;
      last_reheat = st;
      recent_best = energy;
      ++reheats_done;
    }
    T *= exp(-3.0 / (double)(maximum_steps > 1 ? maximum_steps : 1));
    beta = 1.0 / kBoltzmann / (T > 1e-12 ? T : 1e-12);
    if (trace7) {
      double *t = trace7 + 7 * s;
      t[0] = (double)l1;
      t[1] = (double)l2;
      t[2] = accepted;
      t[3] = dE;
      t[4] = e_before;
      t[5] = t_before;
      t[6] = lowest;
    }
  }
  if (state4) {
    state4[0] = (double)st;
    state4[1] = T;
    state4[2] = energy;
    state4[3] = lowest;
  }
  return 0;
}
