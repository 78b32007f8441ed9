/*
 * amca_oracle.c — CPU restatement of AMCA3D's 3-D CA timestep: the plain
 * (uniform-cooling) realm and the FE-coupled remelting realm.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker that the CUDA product
 * is compared against, and the scalar CPU baseline of the benchmark. The
 * product never links it. It is itself checked against the unmodified
 * reference build (oracle/_ref) and the golden fixtures in tests/golden.
 *
 * Reference citations are paths inside the AMCA3D checkout.
 * Build with -ffp-contract=off: the reference's x86-64 build has no FMA, so
 * a*b+c must stay two roundings on every host.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime */
#include "amca_oracle.h"

#include <float.h>
#include <math.h>
#include <time.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_PI 3.14159265358979323846 /* CellularAutomataManager_3D.cpp:24 */
#define THEODORUS 1.732050807568877      /* Octahedron.cpp:13 */

/* ---------------------------------------------------------------------
   libstdc++ std::default_random_engine (minstd_rand0) +
   std::generate_canonical<double,53> + std::normal_distribution (Marsaglia
   polar method), the stream used for critical undercoolings
   (CellularAutomataManager.cpp:174-175, 186). Restated from the published
   algorithms as implemented by GCC's libstdc++ (random.tcc).
   --------------------------------------------------------------------- */
typedef struct {
  uint64_t state;   /* minstd_rand0 state, default seed 1 */
  int saved_avail;  /* normal_distribution keeps the second polar deviate */
  double saved;
} oracle_normal;

static void normal_init(oracle_normal *g) {
  g->state = 1;
  g->saved_avail = 0;
  g->saved = 0.0;
}
static uint64_t minstd_next(oracle_normal *g) {
  g->state = (g->state * 16807u) % 2147483647u;
  return g->state;
}
/* generate_canonical<double, 53>: range R = max-min+1 = 2147483646, so
 * m = max(1, (53 + 30 - 1) / 30) = 2 draws. */
static double canonical(oracle_normal *g) {
  const double r = 2147483646.0;
  double sum = 0.0, tmp = 1.0;
  for (int k = 2; k != 0; --k) {
    sum += (double)(minstd_next(g) - 1u) * tmp;
    tmp *= r; /* r*r = 4611686009837453316 rounds to the same double in long double or double */
  }
  double ret = sum / tmp;
  if (ret >= 1.0) ret = nextafter(1.0, 0.0);
  return ret;
}
static double normal_draw(oracle_normal *g, double mean, double sigma) {
  double ret;
  if (g->saved_avail) {
    g->saved_avail = 0;
    ret = g->saved;
  } else {
    double x, y, r2;
    do {
      x = 2.0 * canonical(g) - 1.0;
      y = 2.0 * canonical(g) - 1.0;
      r2 = x * x + y * y;
    } while (r2 > 1.0 || r2 == 0.0);
    const double mult = sqrt(-2 * log(r2) / r2);
    g->saved = x * mult;
    g->saved_avail = 1;
    ret = y * mult;
  }
  return ret * sigma + mean;
}

void amca_oracle_normal_draws(double mean, double sigma, int n, double *out) {
  oracle_normal g;
  normal_init(&g);
  for (int i = 0; i < n; ++i) out[i] = normal_draw(&g, mean, sigma);
}

/* ---------------------------------------------------------------------
   Orientation: angles from three rand() values
   (CellularAutomataManager_3D.cpp:839-850) and the Bunge ZXZ local->global
   matrix (Octahedron.cpp:282-310).
   --------------------------------------------------------------------- */
void amca_oracle_orientation(int r0, int r1, int r2, double euler[3], double m[9]) {
  double U = (double)r0 / RAND_MAX;
  double V = (double)r1 / RAND_MAX;
  euler[0] = U * 2 * ORACLE_PI;
  euler[1] = acos(2 * V - 1);
  euler[2] = (double)r2 / RAND_MAX * 0.5 * ORACLE_PI;
  amca_oracle_rotation(euler, m);
}

void amca_oracle_rotation(const double euler[3], double m[9]) {
  double ca = cos(euler[0]), sa = sin(euler[0]);
  double cb = cos(euler[1]), sb = sin(euler[1]);
  double cg = cos(euler[2]), sg = sin(euler[2]);
  m[0] = ca * cg - sa * cb * sg;
  m[1] = -ca * sg - sa * cb * cg;
  m[2] = sa * sb;
  m[3] = sa * cg + ca * cb * sg;
  m[4] = -sa * sg + ca * cb * cg;
  m[5] = -ca * sb;
  m[6] = sb * sg;
  m[7] = sb * cg;
  m[8] = cb;
}

/* Global->local coordinates of a cell centre relative to the envelope centre:
 * transMatrixGlobal2Local[3i+j] = transMatrixLocal2Global[i+3j]
 * (Octahedron.cpp:305-308), summed from 0 in component order (:113-121). */
static void to_local(const double m[9], const double gc[3], double c[3]) {
  double cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < 3; i++) {
    cx += gc[i] * m[3 * i + 0];
    cy += gc[i] * m[3 * i + 1];
    cz += gc[i] * m[3 * i + 2];
  }
  c[0] = cx;
  c[1] = cy;
  c[2] = cz;
}

/* Octahedron::cell_is_captured (Octahedron.cpp:99-128). */
int amca_oracle_is_captured(const double m[9], const double gc[3], double length) {
  if (length == 0) return 0;
  double c[3];
  to_local(m, gc, c);
  return fabs(c[0]) + fabs(c[1]) + fabs(c[2]) <= 1.0 * length;
}

/* Octahedron constructor tables (Octahedron.cpp:23-85). */
static const double kNormal[8][3] = {{1, 1, 1},  {-1, 1, 1},  {-1, -1, 1},  {1, -1, 1},
                                     {1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}, {1, -1, -1}};
static const double kCorner[6][3] = {{1, 0, 0}, {0, 1, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
static const int kFaceCorner[8][3] = {{0, 1, 4}, {1, 2, 4}, {2, 3, 4}, {3, 0, 4},
                                      {0, 1, 5}, {1, 2, 5}, {2, 3, 5}, {3, 0, 5}};

static double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */
static double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */

/* Octahedron::capture_cell: decentred new envelope (Octahedron.cpp:134-275).
 * new_info = {dx, dy, dz, L_new}: centre offset (global) and half-diagonal. */
void amca_oracle_capture(const double m[9], const double gc[3], double length, double h, double trunc_coeff,
                         double new_info[4]) {
  new_info[0] = new_info[1] = new_info[2] = new_info[3] = 0.0;
  double c[3];
  to_local(m, gc, c);
  const double cx = c[0], cy = c[1], cz = c[2];
  double interception = fabs(cx) + fabs(cy) + fabs(cz);
  double cc[6][3];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 3; j++) cc[i][j] = kCorner[i][j] * length;
  /* Step 1: face from the octant (:162-176) */
  int quad = 0;
  if (cz >= 0) {
    if (cx >= 0 && cy >= 0) quad = 0;
    else if (cx >= 0 && cy < 0) quad = 3;
    else if (cx < 0 && cy >= 0) quad = 1;
    else if (cx < 0 && cy < 0) quad = 2;
  } else {
    if (cx >= 0 && cy >= 0) quad = 4;
    else if (cx >= 0 && cy < 0) quad = 7;
    else if (cx < 0 && cy >= 0) quad = 5;
    else if (cx < 0 && cy < 0) quad = 6;
  }
  /* Step 2: projection A of the centre on face F (:180-187) */
  double pA[3];
  double perp = length - interception;
  for (int i = 0; i < 3; i++) pA[i] = c[i] + perp * kNormal[quad][i] / 3;
  /* Step 3: nearest corner S1, with the reference's swap order (:191-215) */
  double dist[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 3; i++) {
    const int id = kFaceCorner[quad][i];
    for (int j = 0; j < 3; j++) dist[i] += (pA[j] - cc[id][j]) * ((pA[j] - cc[id][j]));
  }
  int cid[3];
  double mind = dist[0];
  cid[0] = kFaceCorner[quad][0];
  for (int i = 1; i < 3; i++) {
    if (mind > dist[i]) {
      mind = dist[i];
      cid[i] = cid[0];
      cid[0] = kFaceCorner[quad][i];
    } else {
      cid[i] = kFaceCorner[quad][i];
    }
  }
  /* Step 4: projections on S1S2 and S1S3, float sqrt of the norms (:220-245) */
  const int s1 = cid[0], s2 = cid[1], s3 = cid[2];
  double n12 = 0.0, n13 = 0.0, d12 = 0, d13 = 0.0;
  for (int i = 0; i < 3; i++) {
    double s1a = pA[i] - cc[s1][i];
    double s1s2 = cc[s2][i] - cc[s1][i];
    n12 += s1s2 * s1s2;
    d12 += s1a * s1s2;
    double s1s3 = cc[s3][i] - cc[s1][i];
    n13 += s1s3 * s1s3;
    d13 += s1a * s1s3;
  }
  n12 = (double)sqrtf((float)n12);
  n13 = (double)sqrtf((float)n13);
  double I0 = d12 / n12, I1 = n12 - I0;
  double J0 = d13 / n13, J1 = n13 - J0;
  /* Step 5: truncation and new half-diagonal (:248-260) */
  double tv = trunc_coeff * h;
  if (I0 < tv && I1 < tv) {
    I0 = n12 / 2;
    I1 = n13 / 2;
  }
  double L1 = 0.5 * (dmin(I0, tv) + dmin(I1, tv));
  double L2 = 0.5 * (dmin(J0, tv) + dmin(J1, tv));
  double Lnew = (double)sqrtf(2.0f) * (dmax(L1, L2));
  /* Step 6: centre shift along S1, rotated back to global (:266-274) */
  double mag = (length - Lnew);
  for (int i = 0; i < 3; i++) {
    const double comp = mag * cc[s1][i] / (length * THEODORUS);
    for (int j = 0; j < 3; j++) new_info[j] += comp * m[i + j * 3];
  }
  new_info[3] = Lnew;
}

/* ---------------------------------------------------------------------
   The plain CA realm (CellularAutomataManager{,_3D}.cpp).
   --------------------------------------------------------------------- */
typedef struct {
  int nxg, nyg, nzg, nxyg;
  int64_t ncells;
  int32_t *orient, *grain;
  double *dtc;
  /* envelopes (Grain.h:16-22) */
  double *xc, *yc, *zc, *len;
  int32_t *gorient, *gcell;
  int64_t ngrain, gcap;
  /* orientations (Orientation.h) */
  double *euler, *mat;
  int64_t norient, ocap;
  /* active list in ascending envelope id (Grain.cpp:13-18) */
  int32_t *active, *next_active;
  int64_t nactive, acap;
  /* nucleation site list, ascending cell id (CellularAutomataManager.cpp:195-206) */
  int32_t *sites;
  int64_t nsites;
} oracle_state;

static int grow_grains(oracle_state *s, int64_t need) {
  if (need <= s->gcap) return 0;
  int64_t cap = s->gcap ? s->gcap : 1024;
  while (cap < need) cap *= 2;
  double *a = realloc(s->xc, cap * sizeof(double));
  if (!a) return -1;
  s->xc = a;
  a = realloc(s->yc, cap * sizeof(double));
  if (!a) return -1;
  s->yc = a;
  a = realloc(s->zc, cap * sizeof(double));
  if (!a) return -1;
  s->zc = a;
  a = realloc(s->len, cap * sizeof(double));
  if (!a) return -1;
  s->len = a;
  int32_t *b = realloc(s->gorient, cap * sizeof(int32_t));
  if (!b) return -1;
  s->gorient = b;
  b = realloc(s->gcell, cap * sizeof(int32_t));
  if (!b) return -1;
  s->gcell = b;
  s->gcap = cap;
  return 0;
}
static int grow_orient(oracle_state *s, int64_t need) {
  if (need <= s->ocap) return 0;
  int64_t cap = s->ocap ? s->ocap : 256;
  while (cap < need) cap *= 2;
  double *a = realloc(s->euler, cap * 3 * sizeof(double));
  if (!a) return -1;
  s->euler = a;
  a = realloc(s->mat, cap * 9 * sizeof(double));
  if (!a) return -1;
  s->mat = a;
  s->ocap = cap;
  return 0;
}
static int grow_active(oracle_state *s, int64_t need) {
  if (need <= s->acap) return 0;
  int64_t cap = s->acap ? s->acap : 1024;
  while (cap < need) cap *= 2;
  int32_t *a = realloc(s->active, cap * sizeof(int32_t));
  if (!a) return -1;
  s->active = a;
  a = realloc(s->next_active, cap * sizeof(int32_t));
  if (!a) return -1;
  s->next_active = a;
  s->acap = cap;
  return 0;
}

/* get_cell_center (CellularAutomataManager_3D.cpp:877-888), np=1 offsets 0 */
static void cell_center(const oracle_state *s, const amca_oracle_plain_params *p, int64_t id, double c[3]) {
  int K = (int)(id / s->nxyg);
  int I = (int)((id % s->nxyg) % s->nxg);
  int J = (int)((id % s->nxyg) / s->nxg);
  c[0] = p->x0 + p->h * (I - 0.5);
  c[1] = p->y0 + p->h * (J - 0.5);
  c[2] = p->z0 + p->h * (K - 0.5);
}

/* create_new_grain (CellularAutomataManager_3D.cpp:855-871); Grain ctor
 * appends to the active list (Grain.cpp:59-64). */
static int64_t new_grain(oracle_state *s, int32_t cell, int32_t orient, const double c[3], double len) {
  if (grow_grains(s, s->ngrain + 1)) return -1;
  int64_t g = s->ngrain++;
  s->xc[g] = c[0];
  s->yc[g] = c[1];
  s->zc[g] = c[2];
  s->len[g] = len;
  s->gorient[g] = orient;
  s->gcell[g] = cell;
  if (grow_active(s, s->nactive + 1)) return -1;
  s->active[s->nactive++] = (int32_t)g;
  return g;
}

static int cmp_i32(const void *a, const void *b) {
  int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

/* create_nucleation_sites (CellularAutomataManager.cpp:153-213) with
 * get_surface_cells / get_bulk_cells (CellularAutomataManager_3D.cpp:935-1000).
 * The surface scan keeps the reference's "locGhostJ == nxLocGhost_-1" test. */
static int create_sites(oracle_state *s, const amca_oracle_plain_params *p, double density, double mean, double sigma,
                        int surface) {
  int64_t n = 0, cap = 0;
  int32_t *ids = NULL;
  if (surface) {
    cap = 6 * ((int64_t)p->nx * p->ny + (int64_t)p->nx * p->nz + (int64_t)p->ny * p->nz) + 16;
    ids = malloc(cap * sizeof(int32_t));
    if (!ids) return -1;
    for (int64_t i = 0; i < s->ncells; ++i) {
      int K = (int)(i / s->nxyg);
      if (K == 0 || K == s->nzg - 1) continue;
      int I = (int)((i % s->nxyg) % s->nxg);
      if (I == 0 || I == s->nxg - 1) continue;
      int J = (int)((i % s->nxyg) / s->nxg);
      if (J == 0 || J == s->nxg - 1) continue;
      if (K == 1 || K == p->nz)
        if (I != 0 && I != p->nx + 1 && J != 0 && J != p->ny + 1) ids[n++] = (int32_t)i;
      if (I == 1 || I == p->nx)
        if (J != 0 && J != p->ny + 1 && K != 0 && K != p->nz + 1) ids[n++] = (int32_t)i;
      if (J == 1 || J == p->ny)
        if (I != 0 && I != p->nx + 1 && K != 0 && K != p->nz + 1) ids[n++] = (int32_t)i;
    }
  } else {
    cap = (int64_t)p->nx * p->ny * p->nz;
    ids = malloc((cap ? cap : 1) * sizeof(int32_t));
    if (!ids) return -1;
    for (int k = 1; k < s->nzg - 1; ++k)
      for (int j = 1; j < s->nyg - 1; ++j)
        for (int i = 1; i < s->nxg - 1; ++i) ids[n++] = k * s->nxyg + j * s->nxg + i;
  }
  double vpc = surface ? p->h * p->h : p->h * p->h * p->h;
  int numCells = (int)n;
  int numSites = (int)(round(vpc * density * numCells) + 0.5);
  oracle_normal g;
  normal_init(&g);
  int64_t added = 0;
  int32_t *newsites = malloc(((int64_t)numSites + 1) * sizeof(int32_t));
  if (!newsites) {
    free(ids);
    return -1;
  }
  for (int iSite = 0; iSite < numSites; ++iSite) {
    int i = rand() % numCells;
    int cell = ids[i];
    double dT = normal_draw(&g, mean, sigma);
    dT = (dT < 0) ? 0 : dT;
    double cur = s->dtc[cell];
    if (cur < 0) {
      newsites[added++] = cell;
      s->dtc[cell] = dT;
    } else if (dT < cur) {
      s->dtc[cell] = dT;
    }
  }
  /* std::list::sort of the merged list (:206) */
  int32_t *merged = realloc(s->sites, (s->nsites + added + 1) * sizeof(int32_t));
  if (!merged) {
    free(ids);
    free(newsites);
    return -1;
  }
  s->sites = merged;
  memcpy(s->sites + s->nsites, newsites, added * sizeof(int32_t));
  s->nsites += added;
  qsort(s->sites, s->nsites, sizeof(int32_t), cmp_i32);
  free(ids);
  free(newsites);
  return 0;
}

/* ProblemPhysics_RappazGandin1993::compute_growth_velocity (ProblemPhysics.cpp:118-135) */
static double growth_velocity(const amca_oracle_plain_params *p, double time) {
  double T = p->T0 + p->Tdot * time;
  double dT = p->Tm - T;
  double v = 0.0;
  if (dT > 0) {
    v = p->a1 * dT + p->a2 * dT * dT + p->a3 * dT * dT * dT;
    if (v < 0.0) v = 0.0;
  }
  return v;
}

static void free_state(oracle_state *s) {
  free(s->orient);
  free(s->grain);
  free(s->dtc);
  free(s->xc);
  free(s->yc);
  free(s->zc);
  free(s->len);
  free(s->gorient);
  free(s->gcell);
  free(s->euler);
  free(s->mat);
  free(s->active);
  free(s->next_active);
  free(s->sites);
}

int amca_oracle_run_plain(const amca_oracle_plain_params *p, int max_steps, int32_t *orient_out, int32_t *grain_out,
                          double *site_dtc_out, double *euler_out, int64_t euler_cap, amca_oracle_result *res) {
  if (p->nx < 1 || p->ny < 1 || p->nz < 1 || !(p->h > 0)) return -2;
  oracle_state S;
  memset(&S, 0, sizeof S);
  oracle_state *s = &S;
  s->nxg = p->nx + 2;
  s->nyg = p->ny + 2;
  s->nzg = p->nz + 2;
  s->nxyg = s->nxg * s->nyg;
  s->ncells = (int64_t)s->nxyg * s->nzg;
  s->orient = malloc(s->ncells * sizeof(int32_t));
  s->grain = malloc(s->ncells * sizeof(int32_t));
  s->dtc = malloc(s->ncells * sizeof(double));
  if (!s->orient || !s->grain || !s->dtc) {
    free_state(s);
    return -1;
  }
  /* initialize_cells (CellularAutomataManager.cpp:316-326) */
  for (int64_t i = 0; i < s->ncells; ++i) {
    s->orient[i] = -1;
    s->grain[i] = -1;
    s->dtc[i] = -1.0;
  }
  /* initialize_boundaries (CellularAutomataManager_3D.cpp:736-833): ghosts 0 */
  for (int k = 0; k < s->nzg; ++k)
    for (int j = 0; j < s->nyg; ++j)
      for (int i = 0; i < s->nxg; ++i)
        if (k == 0 || k == s->nzg - 1 || j == 0 || j == s->nyg - 1 || i == 0 || i == s->nxg - 1) {
          int64_t id = (int64_t)k * s->nxyg + (int64_t)j * s->nxg + i;
          s->orient[id] = 0;
          s->grain[id] = 0;
        }
  /* ctor srand (CellularAutomataManager_3D.cpp:40), then sites: surface
   * first, then bulk (CellularAutomataManager_3D.cpp:366-379). */
  srand(p->seed);
  if (create_sites(s, p, p->ns, p->mu_s, p->sigma_s, 1) || create_sites(s, p, p->nv, p->mu_v, p->sigma_v, 0)) {
    free_state(s);
    return -1;
  }
  /* global_mapped_grain_ID (CellularAutomataManager.cpp:471-518): with
   * shuffled VTR ids, std::random_shuffle over numGrains = distinct sites
   * draws one rand() per element after the first; the map itself only
   * relabels output, so the oracle just consumes the draws. */
  if (p->shuffle_vtr)
    for (int64_t i = 1; i < s->nsites; ++i) (void)rand();
  int64_t liquid = (int64_t)p->nx * p->ny * p->nz;
  double time = 0.0, dt = 0.0;
  int step = 0;
  int64_t tests = 0;
  int done = 0;
  const double v_floor = 1e-10;
  int32_t nb[26];
  {
    int c = 0;
    for (int k = -1; k < 2; k++)
      for (int j = -1; j < 2; j++)
        for (int i = -1; i < 2; i++) {
          if (k == 0 && j == 0 && i == 0) continue;
          nb[c++] = k * s->nxyg + j * s->nxg + i; /* get_cell_neighbors (:913-925) */
        }
  }
  /* time_integration (CellularAutomataManager.cpp:134-147) */
  while (time < p->final_time && !done && (max_steps < 0 || step < max_steps)) {
    /* --- calculate_time_step (CellularAutomataManager_3D.cpp:441-511) --- */
    /* nucleate_at_nucleation_sites (CellularAutomataManager.cpp:219-297) */
    {
      int64_t w = 0;
      for (int64_t q = 0; q < s->nsites; ++q) {
        int32_t cell = s->sites[q];
        int isLiquid = (s->grain[cell] == -1);
        if (isLiquid) {
          double dTcrit = s->dtc[cell];
          double T = p->T0 + p->Tdot * time; /* compute_cell_temperature (ProblemPhysics.cpp:164-169) */
          double dT = p->Tm - T;
          if (dT > dTcrit) {
            if (grow_orient(s, s->norient + 1)) {
              free_state(s);
              return -1;
            }
            int r0 = rand(), r1 = rand(), r2 = rand();
            int64_t o = s->norient++;
            amca_oracle_orientation(r0, r1, r2, s->euler + 3 * o, s->mat + 9 * o);
            double c[3];
            cell_center(s, p, cell, c);
            int64_t g = new_grain(s, cell, (int32_t)o, c, 0.0);
            if (g < 0) {
              free_state(s);
              return -1;
            }
            s->grain[cell] = (int32_t)g;
            s->orient[cell] = (int32_t)o; /* global id: numCurrentOrientations + local (:1205-1214) */
            liquid--;
            isLiquid = 0;
          }
        }
        if (isLiquid) s->sites[w++] = cell;
        else s->dtc[cell] = 0;
      }
      s->nsites = w;
    }
    double vel = growth_velocity(p, time);
    double maxV = v_floor;
    if (s->nactive > 0 && vel > maxV) maxV = vel;
    {
      double a = p->time_step_factor * p->h / maxV, b = p->max_dt;
      dt = (b < a) ? b : a; /* std::min (:507) */
    }
    /* --- single_integration_step (CellularAutomataManager_3D.cpp:516-669) --- */
    for (int64_t q = 0; q < s->nactive; ++q) {
      int32_t g = s->active[q];
      s->len[g] += dt * vel; /* Grain::grow (Grain.h:27) */
    }
    int64_t nnext = 0;
    for (int64_t q = 0; q < s->nactive; ++q) { /* the list grows while it is walked */
      int32_t g = s->active[q];
      int32_t cell = s->gcell[g];
      int hasNonCaptured = 0;
      const double *m = s->mat + 9 * (int64_t)s->gorient[g];
      for (int n = 0; n < 26; ++n) {
        int32_t nc = cell + nb[n];
        if (s->grain[nc] != -1) continue;
        double cc[3], gc[3];
        cell_center(s, p, nc, cc);
        gc[0] = cc[0] - s->xc[g];
        gc[1] = cc[1] - s->yc[g];
        gc[2] = cc[2] - s->zc[g];
        tests++;
        if (amca_oracle_is_captured(m, gc, s->len[g])) {
          /* CellularAutomataManager_3D::capture_cell (:677-707) */
          double info[4];
          double gcen[3] = {s->xc[g], s->yc[g], s->zc[g]};
          amca_oracle_capture(m, gc, s->len[g], p->h, p->trunc_coeff, info);
          double nc3[3];
          for (int i = 0; i < 3; i++) nc3[i] = info[i] + gcen[i];
          int64_t ng = new_grain(s, nc, s->gorient[g], nc3, info[3]);
          if (ng < 0) {
            free_state(s);
            return -1;
          }
          s->grain[nc] = (int32_t)ng;
          s->orient[nc] = s->gorient[g];
          liquid--;
        } else {
          hasNonCaptured = 1;
        }
      }
      if (hasNonCaptured) {
        if (grow_active(s, nnext + 1)) {
          free_state(s);
          return -1;
        }
        s->next_active[nnext++] = g;
      }
    }
    {
      int32_t *t = s->active;
      s->active = s->next_active;
      s->next_active = t;
      s->nactive = nnext;
    }
    time += dt;
    step++;
    /* get_amount_of_liquid_cells (:2040-2061) */
    if (liquid == 0) done = 1;
  }
  if (orient_out) memcpy(orient_out, s->orient, s->ncells * sizeof(int32_t));
  if (grain_out) memcpy(grain_out, s->grain, s->ncells * sizeof(int32_t));
  if (site_dtc_out) memcpy(site_dtc_out, s->dtc, s->ncells * sizeof(double));
  if (euler_out) {
    int64_t n = s->norient < euler_cap ? s->norient : euler_cap;
    memcpy(euler_out, s->euler, n * 3 * sizeof(double));
  }
  if (res) {
    res->steps = step;
    res->time = time;
    res->last_dt = dt;
    res->num_grains = s->ngrain;
    res->num_orient = s->norient;
    res->liquid_cells = liquid;
    res->active_grains = s->nactive;
    res->tests = tests;
    res->num_sites = 0;
    for (int64_t i = 0; i < s->ncells; ++i)
      if (s->dtc[i] >= 0) res->num_sites++;
  }
  free_state(s);
  return 0;
}

/* =====================================================================
   FE-coupled remelting realm.
   ===================================================================== */

/* std::getline over an in-memory file, with the stream's eof flag: eof is
 * raised when a read reaches the end of the data (no terminating newline, or
 * nothing left to read). */
typedef struct {
  char *buf;
  size_t len, pos;
  int eof;
} line_reader;

static int lr_open(line_reader *L, const char *path) {
  memset(L, 0, sizeof *L);
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  L->buf = malloc((size_t)n + 1);
  if (!L->buf) {
    fclose(f);
    return -1;
  }
  L->len = fread(L->buf, 1, (size_t)n, f);
  L->buf[L->len] = 0;
  fclose(f);
  return 0;
}

/* Returns a NUL-terminated copy of the next line in out (truncated to cap). */
static void lr_getline(line_reader *L, char *out, size_t cap) {
  size_t k = 0;
  if (L->pos >= L->len) {
    L->eof = 1;
    out[0] = 0;
    return;
  }
  while (L->pos < L->len && L->buf[L->pos] != '\n') {
    if (k + 1 < cap) out[k++] = L->buf[L->pos];
    L->pos++;
  }
  if (L->pos < L->len)
    L->pos++; /* the newline */
  else
    L->eof = 1;
  out[k] = 0;
}

/* istringstream >> double / >> int over a line: whitespace-separated
 * tokens converted with strtod / strtol (what libstdc++'s num_get calls). */
static double tok_d(const char **c) {
  char *e;
  double v = strtod(*c, &e);
  *c = e;
  return v;
}
static long tok_l(const char **c) {
  char *e;
  long v = strtol(*c, &e, 10);
  *c = e;
  return v;
}

/* FiniteElementManager replaying frames (FiniteElementManager.h, LoadDataFromFile.cpp). */
typedef struct {
  int nn[3];
  int64_t nnodes, nelem;
  double *coord;           /* Node::coordinates_, 3 per node */
  double *th0, *th1;       /* Node::theta_[0] (newest frame), theta_[1] */
  double *theta;           /* thetaArray_ */
  unsigned char *around;   /* Node::grainAround_ */
  double ts0, ts1, toff;   /* inTimeSeries_[0], [1], inTimeOffset_ */
  double time, dT;         /* time_, dT_ */
  int64_t frames;
  double null_mat;         /* nullMatTemperature_ (= transfers void_temperature) */
  line_reader L;
  int title, subtitle;
  double tscale;
} fe_state;

static void fe_free(fe_state *f) {
  free(f->coord);
  free(f->th0);
  free(f->th1);
  free(f->theta);
  free(f->around);
  free(f->L.buf);
}

/* element e -> its 8 node ids (LoadDataFromFile.cpp:104-131) */
static void fe_elem_nodes(const fe_state *f, int64_t e, int64_t nid[8]) {
  int64_t ncx = f->nn[0] - 1, ncy = f->nn[1] - 1;
  int64_t i = e % ncx, j = (e / ncx) % ncy, k = e / (ncx * ncy);
  int64_t nxy = (int64_t)f->nn[0] * f->nn[1];
  nid[0] = nxy * k + (int64_t)f->nn[0] * j + i;
  nid[1] = nid[0] + 1;
  nid[2] = nid[1] + f->nn[0];
  nid[3] = nid[2] - 1;
  for (int L = 4; L < 8; L++) nid[L] = nid[L - 4] + nxy;
}

/* load_next_step_nodal_data (LoadDataFromFile.cpp:142-191) */
static int fe_load_next(fe_state *f) {
  char line[4096];
  int64_t count = 0;
  while (count < f->subtitle + f->nnodes) {
    if (!f->L.eof)
      lr_getline(&f->L, line, sizeof line);
    else
      return 0;
    if (count == 0 && strcmp(line, "\r") != 0 && strcmp(line, "") != 0) return -1;
    if (count == 3) {
      const char *c = line;
      (void)tok_l(&c);
      (void)tok_l(&c);
      double t0 = tok_d(&c);
      f->ts1 = f->ts0;
      f->ts0 = (t0 - f->toff) * f->tscale;
    }
    if (count >= f->subtitle) {
      const char *c = line;
      (void)tok_d(&c);
      (void)tok_d(&c);
      (void)tok_d(&c);
      double v = tok_d(&c);
      int64_t id = count - f->subtitle;
      f->th1[id] = f->th0[id];
      f->th0[id] = v;
    }
    count++;
  }
  f->frames++;
  return 1;
}

/* load_mesh_and_first_two_steps_results_from_txt_file (LoadDataFromFile.cpp:21-137) */
static int fe_open(fe_state *f, const amca_oracle_remelt_params *p, char *err, int errlen) {
  memset(f, 0, sizeof *f);
  if (lr_open(&f->L, p->frames)) {
    snprintf(err, errlen, "fail to open the specified file %s", p->frames);
    return -1;
  }
  f->title = p->title_lines;
  f->subtitle = p->subtitle_lines;
  f->tscale = p->time_scale;
  char line[4096];
  int count = 0, skip = f->title + f->subtitle;
  double t0 = 0;
  long range[6] = {0, 0, 0, 0, 0, 0};
  while (count < skip) {
    lr_getline(&f->L, line, sizeof line);
    if (count == f->title + 3) {
      const char *c = line;
      (void)tok_l(&c);
      (void)tok_l(&c);
      t0 = tok_d(&c);
      (void)tok_d(&c);
      for (int i = 0; i < 6; i++) range[i] = tok_l(&c);
    }
    count++;
  }
  f->toff = t0;
  f->ts0 = 0.0;
  for (int i = 0; i < 3; i++) f->nn[i] = (int)(range[2 * i + 1] - range[2 * i]) + 1;
  f->nnodes = (int64_t)f->nn[0] * f->nn[1] * f->nn[2];
  if (f->nnodes == 1 || f->nn[0] < 2 || f->nn[1] < 2 || f->nn[2] < 2) {
    snprintf(err, errlen, "fail to read temperature file, please check the file type and the lines of title");
    return -1;
  }
  f->nelem = (int64_t)(f->nn[0] - 1) * (f->nn[1] - 1) * (f->nn[2] - 1);
  f->coord = malloc(3 * f->nnodes * sizeof(double));
  f->th0 = malloc(f->nnodes * sizeof(double));
  f->th1 = malloc(f->nnodes * sizeof(double));
  f->theta = malloc(f->nnodes * sizeof(double));
  f->around = calloc(f->nnodes, 1);
  if (!f->coord || !f->th0 || !f->th1 || !f->theta || !f->around) return -1;
  for (int64_t n = 0; n < f->nnodes; ++n) {
    lr_getline(&f->L, line, sizeof line);
    const char *c = line;
    for (int d = 0; d < 3; d++) {
      double x = tok_d(&c);
      x += p->offset[d];
      x *= p->length_scale;
      f->coord[3 * n + d] = x;
    }
    f->th0[n] = tok_d(&c);
    f->th1[n] = 0.0;
  }
  f->frames = 1;
  if (fe_load_next(f) != 1) {
    snprintf(err, errlen, "fail to read the second frame of the temperature file");
    return -1;
  }
  /* FiniteElementManager::initialize (FiniteElementManager.cpp:147-189) */
  for (int64_t n = 0; n < f->nnodes; ++n) f->theta[n] = f->th1[n];
  return 0;
}

/* pseudo_single_integration_step (LoadDataFromFile.cpp:207-313). Every node
 * is interpolated: the CA reads only grain-around nodes, which are updated
 * on every step in the reference too. */
static int fe_step(fe_state *f, char *err, int errlen) {
  if (f->time == 0) f->time = f->ts1;
  f->time += f->dT;
  while (f->time >= f->ts0) {
    int r = fe_load_next(f);
    if (r < 0) {
      snprintf(err, errlen, "fail to read next step temperature file, please check title of line");
      return -1;
    }
    if (r == 0) return 0;
  }
  double ratio = (f->time - f->ts1) / (f->ts0 - f->ts1);
  if (ratio < 0.0) {
    snprintf(err, errlen, "time ratio error: timeRatio is less then 0");
    return -1;
  }
  for (int64_t n = 0; n < f->nnodes; ++n) {
    if (f->th0[n] <= f->null_mat)
      f->theta[n] = f->null_mat;
    else if (f->th1[n] <= f->null_mat)
      f->theta[n] = f->th0[n];
    else
      f->theta[n] = ratio * (f->th0[n] - f->th1[n]) + f->th1[n];
  }
  return 1;
}

/* ---------------------------------------------------------------------
   MapVoxelManager (MapVoxelManager.cpp)
   --------------------------------------------------------------------- */
static double mv_min(double a, double b) { return ((a) < (b)) ? (a) : (b); } /* __min (:11) */
static double mv_max(double a, double b) { return ((a) > (b)) ? (a) : (b); } /* __max (:10) */

/* get_cell_xyz_min_max (:262-289) */
static void elem_range(const fe_state *f, int64_t e, double r[6]) {
  int64_t nid[8];
  fe_elem_nodes(f, e, nid);
  for (int i = 0; i < 3; i++) {
    r[2 * i] = 1.0e8;
    r[2 * i + 1] = -1.0e8;
  }
  for (int n = 0; n < 8; n++) {
    const double *c = f->coord + 3 * nid[n];
    for (int d = 0; d < 3; d++) {
      r[2 * d] = mv_min(r[2 * d], c[d]);
      r[2 * d + 1] = mv_max(r[2 * d + 1], c[d]);
    }
  }
}

/* is_in_element (:487-699): Newton-Raphson for the parametric coordinates of
 * a point in a trilinear hex, in the reference's operation order. x/y/z hold
 * 0.125 * (node - node0). */
static int in_element(const double X[8], const double Y[8], const double Z[8], double xp, double yp, double zp,
                      double tol, int max_iter, double para[3]) {
  const double *x = X, *y = Y, *z = Z;
  double j[9], f[3], s[8];
  double xinew = 0.5, etanew = 0.5, zetanew = 0.5;
  double xi = 0.5, eta = 0.5, zeta = 0.5;
  double d[3] = {1.0, 1.0, 1.0};
  int i = 0;
  do {
    j[0] = -(1.0 - eta) * (1.0 - zeta) * x[1] - (1.0 + eta) * (1.0 - zeta) * x[2] +
           (1.0 + eta) * (1.0 - zeta) * x[3] + (1.0 - eta) * (1.0 + zeta) * x[4] -
           (1.0 - eta) * (1.0 + zeta) * x[5] - (1.0 + eta) * (1.0 + zeta) * x[6] +
           (1.0 + eta) * (1.0 + zeta) * x[7];
    j[1] = (1.0 + xi) * (1.0 - zeta) * x[1] - (1.0 + xi) * (1.0 - zeta) * x[2] - (1.0 - xi) * (1.0 - zeta) * x[3] +
           (1.0 - xi) * (1.0 + zeta) * x[4] + (1.0 + xi) * (1.0 + zeta) * x[5] - (1.0 + xi) * (1.0 + zeta) * x[6] -
           (1.0 - xi) * (1.0 + zeta) * x[7];
    j[2] = (1.0 - eta) * (1.0 + xi) * x[1] + (1.0 + eta) * (1.0 + xi) * x[2] + (1.0 + eta) * (1.0 - xi) * x[3] -
           (1.0 - eta) * (1.0 - xi) * x[4] - (1.0 - eta) * (1.0 + xi) * x[5] - (1.0 + eta) * (1.0 + xi) * x[6] -
           (1.0 + eta) * (1.0 - xi) * x[7];
    j[3] = -(1.0 - eta) * (1.0 - zeta) * y[1] - (1.0 + eta) * (1.0 - zeta) * y[2] +
           (1.0 + eta) * (1.0 - zeta) * y[3] + (1.0 - eta) * (1.0 + zeta) * y[4] -
           (1.0 - eta) * (1.0 + zeta) * y[5] - (1.0 + eta) * (1.0 + zeta) * y[6] +
           (1.0 + eta) * (1.0 + zeta) * y[7];
    j[4] = (1.0 + xi) * (1.0 - zeta) * y[1] - (1.0 + xi) * (1.0 - zeta) * y[2] - (1.0 - xi) * (1.0 - zeta) * y[3] +
           (1.0 - xi) * (1.0 + zeta) * y[4] + (1.0 + xi) * (1.0 + zeta) * y[5] - (1.0 + xi) * (1.0 + zeta) * y[6] -
           (1.0 - xi) * (1.0 + zeta) * y[7];
    j[5] = (1.0 - eta) * (1.0 + xi) * y[1] + (1.0 + eta) * (1.0 + xi) * y[2] + (1.0 + eta) * (1.0 - xi) * y[3] -
           (1.0 - eta) * (1.0 - xi) * y[4] - (1.0 - eta) * (1.0 + xi) * y[5] - (1.0 + eta) * (1.0 + xi) * y[6] -
           (1.0 + eta) * (1.0 - xi) * y[7];
    j[6] = -(1.0 - eta) * (1.0 - zeta) * z[1] - (1.0 + eta) * (1.0 - zeta) * z[2] +
           (1.0 + eta) * (1.0 - zeta) * z[3] + (1.0 - eta) * (1.0 + zeta) * z[4] -
           (1.0 - eta) * (1.0 + zeta) * z[5] - (1.0 + eta) * (1.0 + zeta) * z[6] +
           (1.0 + eta) * (1.0 + zeta) * z[7];
    j[7] = (1.0 + xi) * (1.0 - zeta) * z[1] - (1.0 + xi) * (1.0 - zeta) * z[2] - (1.0 - xi) * (1.0 - zeta) * z[3] +
           (1.0 - xi) * (1.0 + zeta) * z[4] + (1.0 + xi) * (1.0 + zeta) * z[5] - (1.0 + xi) * (1.0 + zeta) * z[6] -
           (1.0 - xi) * (1.0 + zeta) * z[7];
    j[8] = (1.0 - eta) * (1.0 + xi) * z[1] + (1.0 + eta) * (1.0 + xi) * z[2] + (1.0 + eta) * (1.0 - xi) * z[3] -
           (1.0 - eta) * (1.0 - xi) * z[4] - (1.0 - eta) * (1.0 + xi) * z[5] - (1.0 + eta) * (1.0 + xi) * z[6] -
           (1.0 + eta) * (1.0 - xi) * z[7];
    double jdet = -(j[2] * j[4] * j[6]) + j[1] * j[5] * j[6] + j[2] * j[3] * j[7] - j[0] * j[5] * j[7] -
                  j[1] * j[3] * j[8] + j[0] * j[4] * j[8];
    if (!jdet) {
      i = max_iter;
      break;
    }
    s[0] = (1.0 - eta) * (1.0 - xi) * (1.0 - zeta);
    s[1] = (1.0 - eta) * (1.0 + xi) * (1.0 - zeta);
    s[2] = (1.0 + eta) * (1.0 + xi) * (1.0 - zeta);
    s[3] = (1.0 + eta) * (1.0 - xi) * (1.0 - zeta);
    s[4] = (1.0 - eta) * (1.0 - xi) * (1.0 + zeta);
    s[5] = (1.0 - eta) * (1.0 + xi) * (1.0 + zeta);
    s[6] = (1.0 + eta) * (1.0 + xi) * (1.0 + zeta);
    s[7] = (1.0 + eta) * (1.0 - xi) * (1.0 + zeta);
    f[0] = xp - s[1] * x[1] - s[2] * x[2] - s[3] * x[3] - s[4] * x[4] - s[5] * x[5] - s[6] * x[6] - s[7] * x[7];
    f[1] = yp - s[1] * y[1] - s[2] * y[2] - s[3] * y[3] - s[4] * y[4] - s[5] * y[5] - s[6] * y[6] - s[7] * y[7];
    f[2] = zp - s[1] * z[1] - s[2] * z[2] - s[3] * z[3] - s[4] * z[4] - s[5] * z[5] - s[6] * z[6] - s[7] * z[7];
    xinew = (jdet * xi + f[2] * (j[2] * j[4] - j[1] * j[5]) + f[1] * (j[1] * j[8] - j[2] * j[7]) +
             f[0] * (j[5] * j[7] - j[4] * j[8])) /
            jdet;
    etanew = (eta * jdet + f[2] * (j[0] * j[5] - j[2] * j[3]) + f[1] * (j[2] * j[6] - j[0] * j[8]) +
              f[0] * (j[3] * j[8] - j[5] * j[6])) /
             jdet;
    zetanew = (jdet * zeta + f[2] * (j[1] * j[3] - j[0] * j[4]) + f[1] * (j[0] * j[7] - j[1] * j[6]) +
               f[0] * (j[4] * j[6] - j[3] * j[7])) /
              jdet;
    d[0] = xinew - xi;
    d[1] = etanew - eta;
    d[2] = zetanew - zeta;
    xi = xinew;
    eta = etanew;
    zeta = zetanew;
  } while (!(fabs(0.0 + d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) < tol) && ++i < max_iter);
  para[0] = para[1] = para[2] = DBL_MAX;
  double dist = DBL_MAX;
  if (i < max_iter) {
    para[0] = xinew;
    para[1] = etanew;
    para[2] = zetanew;
    dist = 0;
    for (int c = 0; c < 3; c++) {
      if (para[c] > 1.0 && para[c] < 1.000001) para[c] = 1.0;
      if (para[c] < -1.0 && para[c] > -1.000001) para[c] = -1.0;
    }
    for (int c = 0; c < 3; c++) /* parametric_distance (:726-741) */
      if (dist < fabs(para[c])) dist = fabs(para[c]);
  }
  return !(dist > 1.0);
}

int amca_oracle_is_in_element(const double node_xyz[24], const double point[3], double tolerance, int max_iter,
                              double para[3]) {
  double x[8], y[8], z[8];
  x[0] = y[0] = z[0] = 0.0;
  const double *o = node_xyz;
  for (int n = 1; n < 8; n++) {
    x[n] = 0.125 * (node_xyz[3 * n] - o[0]);
    y[n] = 0.125 * (node_xyz[3 * n + 1] - o[1]);
    z[n] = 0.125 * (node_xyz[3 * n + 2] - o[2]);
  }
  return in_element(x, y, z, point[0] - o[0], point[1] - o[1], point[2] - o[2], tolerance, max_iter, para);
}

/* execute_with_focus_on_CA_region (:140-164): CA-region bounds, bins,
 * element attachment, voxel tagging. tag/pc are over the ghost-inclusive
 * voxels; unmatched voxels keep tag -1 and parametric coordinates -2. */
static int map_voxels(fe_state *f, const amca_oracle_remelt_params *p, int32_t *tag, double *pc, char *err,
                      int errlen) {
  const int nxg = p->nx + 2, nyg = p->ny + 2, nzg = p->nz + 2;
  const int64_t nxyg = (int64_t)nxg * nyg, nvox = nxyg * nzg;
  const double h = p->h;
  for (int64_t v = 0; v < nvox; ++v) {
    tag[v] = -1;
    pc[3 * v] = pc[3 * v + 1] = pc[3 * v + 2] = -2;
  }
  /* get_CA_domain_xyz_min_max (:198-256), np=1 start offsets 0 */
  double mm[6], cur[6];
  mm[0] = (0 - 1) * h + p->x0;
  mm[2] = (0 - 1) * h + p->y0;
  mm[4] = (0 - 1) * h + p->z0;
  mm[1] = mm[0] + nxg * h;
  mm[3] = mm[2] + nyg * h;
  mm[5] = mm[4] + nzg * h;
  for (int c = 0; c < 6; c++) cur[c] = mm[c];
  for (int64_t e = 0; e < f->nelem; ++e) {
    int64_t nid[8];
    fe_elem_nodes(f, e, nid);
    int overlap = 0;
    for (int n = 0; n < 8; n++) {
      const double *c = f->coord + 3 * nid[n];
      if (c[0] >= mm[0] && c[0] <= mm[1] && c[1] >= mm[2] && c[1] <= mm[3] && c[2] >= mm[4] && c[2] <= mm[5]) {
        overlap = 1;
        break;
      }
    }
    if (overlap) {
      double r[6];
      elem_range(f, e, r);
      for (int d = 0; d < 3; d++) {
        cur[2 * d] = mv_min(cur[2 * d], r[2 * d]);
        cur[2 * d + 1] = mv_max(cur[2 * d + 1], r[2 * d + 1]);
      }
    }
  }
  for (int c = 0; c < 6; c++) mm[c] = cur[c];
  double dBin[3];
  int numBin[3];
  for (int i = 0; i < 3; i++) {
    dBin[i] = p->bin[i] * h;
    numBin[i] = (int)ceil((mm[i * 2 + 1] - mm[i * 2]) / dBin[i]);
  }
  int64_t nbins = (int64_t)numBin[0] * numBin[1] * numBin[2];
  /* attach_elements (:294-352) into CSR lists, push order kept */
  int64_t *start = calloc(nbins + 1, sizeof(int64_t));
  if (!start) return -1;
  for (int pass = 0; pass < 2; ++pass) {
    int64_t *fill = NULL;
    int32_t *list = NULL;
    if (pass == 1) {
      for (int64_t b = 0; b < nbins; ++b) start[b + 1] += start[b];
      fill = malloc((nbins + 1) * sizeof(int64_t));
      list = malloc((start[nbins] + 1) * sizeof(int32_t));
      if (!fill || !list) {
        free(fill);
        free(list);
        free(start);
        return -1;
      }
      memcpy(fill, start, nbins * sizeof(int64_t));
    }
    for (int64_t e = 0; e < f->nelem; ++e) {
      double r[6];
      elem_range(f, e, r);
      int inside = 1;
      for (int c = 0; c < 3; c++)
        if (r[c * 2] < mm[c * 2] || r[c * 2 + 1] > mm[c * 2 + 1]) {
          inside = 0;
          break;
        }
      if (!inside) continue;
      if (pass == 0) {
        int64_t nid[8];
        fe_elem_nodes(f, e, nid);
        for (int n = 0; n < 8; n++) f->around[nid[n]] = 1;
      }
      int imin = (int)floor((r[0] - mm[0]) / dBin[0]);
      int imax = (int)ceil((r[1] - mm[0]) / dBin[0]);
      int jmin = (int)floor((r[2] - mm[2]) / dBin[1]);
      int jmax = (int)ceil((r[3] - mm[2]) / dBin[1]);
      int kmin = (int)floor((r[4] - mm[4]) / dBin[2]);
      int kmax = (int)ceil((r[5] - mm[4]) / dBin[2]);
      for (int kk = kmin; kk < kmax; kk++)
        for (int jj = jmin; jj < jmax; jj++)
          for (int ii = imin; ii < imax; ii++) {
            int64_t ind = ii + (int64_t)jj * numBin[0] + (int64_t)kk * numBin[0] * numBin[1];
            if (ind < 0 || ind >= nbins) continue; /* cannot happen for elements inside the bounds */
            if (pass == 0)
              start[ind + 1]++;
            else
              list[fill[ind]++] = (int32_t)e;
          }
    }
    if (pass == 1) {
      /* tag_voxels (:357-482) */
      double origin[3] = {(0 - 0.5) * h + p->x0, (0 - 0.5) * h + p->y0, (0 - 0.5) * h + p->z0};
      int found_any = 0;
      for (int64_t v = 0; v < nvox; ++v) {
        int idx[3], mmb[6];
        idx[2] = (int)(v / nxyg);
        idx[1] = (int)((v % nxyg) / nxg);
        idx[0] = (int)((v % nxyg) % nxg);
        double cv[3];
        int out = 0;
        for (int c = 0; c < 3; c++) {
          cv[c] = origin[c] + idx[c] * h;
          if (cv[c] < mm[2 * c] || cv[c] > mm[2 * c + 1]) {
            out = 1;
            break;
          }
          double dist = cv[c] - mm[2 * c];
          mmb[2 * c] = (int)floor(dist / dBin[c]);
          mmb[2 * c + 1] = (int)ceil(dist / dBin[c]);
        }
        if (out) continue;
        for (int c = 0; c < 3; c++) {
          int *lo = &mmb[2 * c], *hi = &mmb[2 * c + 1];
          if (*lo == *hi && *lo > 0 && *hi < numBin[c]) {
            *lo -= 1;
            *hi += 1;
          } else if (*hi == 0) {
            *hi = 1;
          } else if (*hi == numBin[c]) {
            if (*lo > 0) *lo -= 1;
          }
        }
        int got = 0;
        for (int kk = mmb[4]; kk < mmb[5] && !got; kk++)
          for (int jj = mmb[2]; jj < mmb[3] && !got; jj++)
            for (int ii = mmb[0]; ii < mmb[1] && !got; ii++) {
              int64_t ind = ii + (int64_t)jj * numBin[0] + (int64_t)kk * numBin[0] * numBin[1];
              for (int64_t q = start[ind]; q < start[ind + 1]; ++q) {
                int64_t e = list[q];
                double r[6];
                elem_range(f, e, r);
                if (cv[0] < r[0] || cv[0] > r[1] || cv[1] < r[2] || cv[1] > r[3] || cv[2] < r[4] || cv[2] > r[5])
                  continue;
                int64_t nid[8];
                fe_elem_nodes(f, e, nid);
                double X[8], Y[8], Z[8], para[3];
                const double *o = f->coord + 3 * nid[0];
                X[0] = Y[0] = Z[0] = 0.0;
                for (int n = 1; n < 8; n++) {
                  const double *c = f->coord + 3 * nid[n];
                  X[n] = 0.125 * (c[0] - o[0]);
                  Y[n] = 0.125 * (c[1] - o[1]);
                  Z[n] = 0.125 * (c[2] - o[2]);
                }
                if (in_element(X, Y, Z, cv[0] - o[0], cv[1] - o[1], cv[2] - o[2], p->tolerance, p->max_iter,
                               para)) {
                  tag[v] = (int32_t)e;
                  pc[3 * v] = para[0];
                  pc[3 * v + 1] = para[1];
                  pc[3 * v + 2] = para[2];
                  got = 1;
                  found_any = 1;
                  break;
                }
              }
            }
      }
      free(fill);
      free(list);
      free(start);
      if (!found_any) {
        snprintf(err, errlen, "Error: a proc has no corrsponding FEM mesh!!");
        return -1;
      }
    }
  }
  return 0;
}

/* evaluate_temperature (:746-799) */
static int eval_temperature(const fe_state *f, const int32_t *tag, const double *pc, int64_t v, double void_t,
                            double *T) {
  double nullMat = void_t + 0.00001;
  int32_t e = tag[v];
  if (e < 0) return 0;
  int64_t nid[8];
  fe_elem_nodes(f, e, nid);
  for (int i = 0; i < 8; i++)
    if (f->theta[nid[i]] < nullMat) return 0;
  double xi = pc[3 * v], eta = pc[3 * v + 1], zeta = pc[3 * v + 2];
  double s[8];
  s[0] = 0.125 * (1.0 - eta) * (1.0 - xi) * (1.0 - zeta);
  s[1] = 0.125 * (1.0 - eta) * (1.0 + xi) * (1.0 - zeta);
  s[2] = 0.125 * (1.0 + eta) * (1.0 + xi) * (1.0 - zeta);
  s[3] = 0.125 * (1.0 + eta) * (1.0 - xi) * (1.0 - zeta);
  s[4] = 0.125 * (1.0 - eta) * (1.0 - xi) * (1.0 + zeta);
  s[5] = 0.125 * (1.0 - eta) * (1.0 + xi) * (1.0 + zeta);
  s[6] = 0.125 * (1.0 + eta) * (1.0 + xi) * (1.0 + zeta);
  s[7] = 0.125 * (1.0 + eta) * (1.0 - xi) * (1.0 + zeta);
  double t = 0.0;
  for (int i = 0; i < 8; i++) t += s[i] * f->theta[nid[i]];
  *T = t;
  return 1;
}

/* ---------------------------------------------------------------------
   CellularAutomataManager_3DRemelting
   --------------------------------------------------------------------- */
typedef struct {
  oracle_state s;          /* cell ids, grains, orientations, sites */
  double *T;               /* cellTemperature_ */
  uint8_t *cooling, *melted, *flag; /* cooling_, hasBeenMelted_, cellLiquidNeigh */
  int32_t *tag;            /* MapVoxelManager elementTagList_ */
  double *pc;              /* parCoordsList_ */
  amca_oracle_plain_params g; /* grid fields for the shared helpers */
} remelt_state;

static void remelt_free(remelt_state *r) {
  free_state(&r->s);
  free(r->T);
  free(r->cooling);
  free(r->melted);
  free(r->flag);
  free(r->tag);
  free(r->pc);
}

/* ProblemPhysics_RappazGandin1993::compute_growth_velocity_with_temperature_input
 * (ProblemPhysics.cpp:142-158), libm pow as in the reference */
static double remelt_velocity(const amca_oracle_remelt_params *p, double T) {
  double dT = p->Tm - T;
  double v = 0.0;
  if (dT > 0) {
    v = p->a1 * pow(dT, p->b1) + p->a2 * pow(dT, p->b2) + p->a3 * pow(dT, p->b3);
    if (v < 0.0) v = 0.0;
  }
  return v;
}

/* a grain that is not on the active list (Grain(this, false)) */
static int64_t remelt_new_grain(oracle_state *s, int32_t cell, int32_t orient, const double c[3], double len) {
  if (grow_grains(s, s->ngrain + 1)) return -1;
  int64_t g = s->ngrain++;
  s->xc[g] = c[0];
  s->yc[g] = c[1];
  s->zc[g] = c[2];
  s->len[g] = len;
  s->gorient[g] = orient;
  s->gcell[g] = cell;
  return g;
}

static int64_t remelt_new_orientation(oracle_state *s) {
  if (grow_orient(s, s->norient + 1)) return -1;
  int r0 = rand(), r1 = rand(), r2 = rand(); /* get_random_orientation_angle (CellularAutomataManager_3D.cpp:839-850) */
  int64_t o = s->norient++;
  amca_oracle_orientation(r0, r1, r2, s->euler + 3 * o, s->mat + 9 * o);
  return o;
}

static int is_ghost_cell(const oracle_state *s, int64_t id) { /* np=1: cell_is_ghost == cell_is_global_ghost */
  int K = (int)(id / s->nxyg), I = (int)((id % s->nxyg) % s->nxg), J = (int)((id % s->nxyg) / s->nxg);
  return I == 0 || I == s->nxg - 1 || J == 0 || J == s->nyg - 1 || K == 0 || K == s->nzg - 1;
}

static void shuffle_draws(int64_t n) { /* std::random_shuffle: one rand() per element after the first */
  for (int64_t i = 1; i < n; ++i) (void)rand();
}

/* load_microstructure_information (CellularAutomataManager_3DRemelting.cpp:164-307)
 * + retrieve_grain_information_before_simulation (:312-332). */
static int remelt_load(remelt_state *r, const amca_oracle_remelt_params *p, int64_t *expected, char *err, int errlen) {
  oracle_state *s = &r->s;
  const char *path = p->microstructure;
  char fname[4096];
  const char *dot = strrchr(path, '.');
  size_t stem = dot ? (size_t)(dot - path) : strlen(path);
  if (stem > sizeof fname - 8) stem = sizeof fname - 8;
  memcpy(fname, path, stem);
  strcpy(fname + stem, "0.txt");
  line_reader L;
  if (lr_open(&L, fname)) {
    snprintf(err, errlen, "fail to open the specified file %s", fname);
    return -1;
  }
  char line[4096];
  lr_getline(&L, line, sizeof line);
  lr_getline(&L, line, sizeof line);
  const char *c = line;
  long ncells = tok_l(&c), norient = tok_l(&c), ngrains = tok_l(&c), nexp = tok_l(&c);
  *expected = nexp;
  if (!p->nucleation && p->shuffle_vtr) shuffle_draws(nexp);
  if (ncells != s->ncells) {
    snprintf(err, errlen, "Error : microstructure information file is not fit the current domain size");
    free(L.buf);
    return -1;
  }
  lr_getline(&L, line, sizeof line);
  for (long n = 0; n < ncells;) {
    if (L.eof) break;
    lr_getline(&L, line, sizeof line);
    if (!line[0]) continue;
    c = line;
    long id = tok_l(&c), g = tok_l(&c), o = tok_l(&c), m = tok_l(&c);
    double dt = tok_d(&c);
    if (id >= 0 && id < s->ncells) {
      s->grain[id] = (int32_t)g;
      s->orient[id] = (int32_t)o;
      r->melted[id] = (uint8_t)(m != 0);
      if (p->load_seeds && dt > -1) {
        s->dtc[id] = dt;
        int32_t *ns = realloc(s->sites, (s->nsites + 1) * sizeof(int32_t));
        if (!ns) {
          free(L.buf);
          return -1;
        }
        s->sites = ns;
        s->sites[s->nsites++] = (int32_t)id;
      }
    }
    n++;
  }
  lr_getline(&L, line, sizeof line);
  if (grow_orient(s, norient + 1)) {
    free(L.buf);
    return -1;
  }
  for (long n = 0; n < norient;) {
    if (L.eof) break;
    lr_getline(&L, line, sizeof line);
    if (!line[0]) continue;
    c = line;
    long id = tok_l(&c);
    double e[3];
    e[0] = tok_d(&c);
    e[1] = tok_d(&c);
    e[2] = tok_d(&c);
    if (id != n) {
      snprintf(err, errlen, "orientation ids in the microstructure file must be 0..n-1 in order");
      free(L.buf);
      return -1;
    }
    memcpy(s->euler + 3 * n, e, sizeof e);
    amca_oracle_rotation(e, s->mat + 9 * n);
    n++;
  }
  s->norient = norient;
  lr_getline(&L, line, sizeof line);
  for (long n = 0; n < ngrains;) {
    if (L.eof) break;
    lr_getline(&L, line, sizeof line);
    if (!line[0]) continue;
    c = line;
    (void)tok_l(&c);
    long cell = tok_l(&c);
    (void)tok_d(&c);
    (void)tok_d(&c);
    (void)tok_d(&c);
    long o = tok_l(&c);
    double cc[3];
    cell_center(s, &r->g, cell, cc);
    if (remelt_new_grain(s, (int32_t)cell, (int32_t)o, cc, 0.0) < 0) {
      free(L.buf);
      return -1;
    }
    n++;
  }
  free(L.buf);
  for (int64_t i = 0; i < s->ncells; ++i) {
    if (is_ghost_cell(s, i)) {
      s->orient[i] = -1;
      continue;
    }
    if (s->orient[i] > -1) continue;
    int32_t g = s->grain[i];
    if (g < 0 || g >= s->ngrain) {
      snprintf(err, errlen, "cell %lld has neither an orientation nor a grain", (long long)i);
      return -1;
    }
    s->orient[i] = s->gorient[g];
  }
  return 0;
}

static int dump_put(FILE *f, const void *p, size_t n) { return (n && fwrite(p, 1, n, f) != n) ? -1 : 0; }

/* One record in the layout of oracle/ref_probe/state_dump.cpp. */
static int remelt_dump(const remelt_state *r, const fe_state *fe, FILE *f, int first, int step, double time, double dt,
                       double maxdt) {
  const oracle_state *s = &r->s;
  int32_t n = (int32_t)s->ncells;
  int rc = 0;
  if (first) {
    rc |= dump_put(f, "AMCT", 4);
    rc |= dump_put(f, &n, 4);
    rc |= dump_put(f, r->tag, 4 * (size_t)n);
    rc |= dump_put(f, r->pc, 24 * (size_t)n);
  }
  int32_t hdr[4] = {n, (int32_t)s->ngrain, (int32_t)s->norient, (int32_t)fe->nnodes};
  double tt[3] = {time, dt, maxdt};
  rc |= dump_put(f, "AMCD", 4);
  rc |= dump_put(f, &step, 4);
  rc |= dump_put(f, tt, 24);
  rc |= dump_put(f, hdr, 16);
  rc |= dump_put(f, s->orient, 4 * (size_t)n);
  rc |= dump_put(f, s->grain, 4 * (size_t)n);
  rc |= dump_put(f, r->T, 8 * (size_t)n);
  rc |= dump_put(f, r->cooling, n);
  rc |= dump_put(f, r->melted, n);
  rc |= dump_put(f, r->flag, n);
  for (int64_t g = 0; g < s->ngrain; ++g) {
    int32_t rec[3] = {(int32_t)g, s->gcell[g], s->gorient[g]};
    uint8_t act = 0;
    double geo[4] = {s->xc[g], s->yc[g], s->zc[g], s->len[g]};
    rc |= dump_put(f, rec, 12);
    rc |= dump_put(f, &act, 1);
    rc |= dump_put(f, geo, 32);
  }
  rc |= dump_put(f, s->euler, 24 * (size_t)s->norient);
  rc |= dump_put(f, fe->theta, 8 * (size_t)fe->nnodes);
  return rc;
}

int amca_oracle_run_remelt(const amca_oracle_remelt_params *p, int max_steps, const char *dump_path,
                           int32_t *orient_out, int32_t *grain_out, double *temp_out, uint8_t *melted_out,
                           uint8_t *cooling_out, uint8_t *flag_out, amca_oracle_remelt_result *res, char *err,
                           int errlen) {
  char dummy_err[8];
  if (!err || errlen <= 0) {
    err = dummy_err;
    errlen = (int)sizeof dummy_err;
  }
  err[0] = 0;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1 || !(p->h > 0) || !p->frames) {
    snprintf(err, errlen, "bad grid or missing frames");
    return -2;
  }
  remelt_state R;
  memset(&R, 0, sizeof R);
  oracle_state *s = &R.s;
  R.g.nx = p->nx;
  R.g.ny = p->ny;
  R.g.nz = p->nz;
  R.g.x0 = p->x0;
  R.g.y0 = p->y0;
  R.g.z0 = p->z0;
  R.g.h = p->h;
  s->nxg = p->nx + 2;
  s->nyg = p->ny + 2;
  s->nzg = p->nz + 2;
  s->nxyg = s->nxg * s->nyg;
  s->ncells = (int64_t)s->nxyg * s->nzg;
  const int64_t N = s->ncells;
  s->orient = malloc(N * sizeof(int32_t));
  s->grain = malloc(N * sizeof(int32_t));
  s->dtc = malloc(N * sizeof(double));
  R.T = malloc(N * sizeof(double));
  R.cooling = calloc(N, 1);
  R.melted = calloc(N, 1);
  R.flag = calloc(N, 1);
  R.tag = malloc(N * sizeof(int32_t));
  R.pc = malloc(3 * N * sizeof(double));
  fe_state FE;
  memset(&FE, 0, sizeof FE);
  FILE *dump = NULL;
  int rc = -1;
  if (!s->orient || !s->grain || !s->dtc || !R.T || !R.cooling || !R.melted || !R.flag || !R.tag || !R.pc) goto done;
  const double nullMatTemp = -1.0; /* CellularAutomataManager_3DRemelting ctor (:29) */
  const double void_t = p->void_temperature;

  /* ---- CafeSolver::load/initialize (CafeSolver.cpp:40-154) ---- */
  if (fe_open(&FE, p, err, errlen)) goto done;
  FE.null_mat = void_t;
  /* ctor srand (CellularAutomataManager_3D.cpp:40) */
  srand(p->seed);
  /* setup_cells: initialize_cells + initialize_boundaries */
  for (int64_t i = 0; i < N; ++i) {
    s->orient[i] = -1;
    s->grain[i] = -1;
    s->dtc[i] = -1.0;
    if (is_ghost_cell(s, i)) s->orient[i] = s->grain[i] = 0;
  }
  const double cutoff = p->cutoff_factor * p->h;
  for (int64_t i = 0; i < N; ++i) {
    R.T[i] = nullMatTemp;
    R.cooling[i] = 0;
    R.flag[i] = 0;
    R.melted[i] = (uint8_t)(p->initial_melted ? 1 : 0);
  }
  int64_t existing = 0;
  if (!p->microstructure) {
    /* random_microstructure_information (CellularAutomataManager_3D.cpp:1929-1984) */
    for (int64_t i = 0; i < N; ++i) {
      if (is_ghost_cell(s, i)) {
        s->grain[i] = -1;
        s->orient[i] = -1;
        continue;
      }
      int64_t o = remelt_new_orientation(s);
      double c[3];
      cell_center(s, &R.g, i, c);
      int64_t g = o < 0 ? -1 : remelt_new_grain(s, (int32_t)i, (int32_t)o, c, 0.0);
      if (g < 0) goto done;
      s->grain[i] = (int32_t)g;
      s->orient[i] = (int32_t)o;
    }
    if (p->shuffle_vtr) shuffle_draws(N);
  } else if (remelt_load(&R, p, &existing, err, errlen)) {
    goto done;
  }
  if (p->nucleation) {
    if (create_sites(s, &R.g, p->ns, p->mu_s, p->sigma_s, 1) || create_sites(s, &R.g, p->nv, p->mu_v, p->sigma_v, 0))
      goto done;
    if (p->shuffle_vtr) { /* global_mapped_grain_ID_plus (:873-931) */
      int64_t surf = ((int64_t)p->nx * p->ny + (int64_t)p->nx * (p->nz - 2) + (int64_t)(p->ny - 2) * (p->nz - 2)) * 2;
      int64_t bulk = (int64_t)p->nx * p->ny * p->nz;
      int ss = (int)(round(p->ns * surf * (p->h * p->h)) + 0.5);
      int sb = (int)(round(p->nv * bulk * (p->h * p->h * p->h)) + 0.5);
      shuffle_draws((int64_t)ss + sb + existing);
    }
  }
  if (map_voxels(&FE, p, R.tag, R.pc, err, errlen)) goto done;
  if (dump_path) {
    dump = fopen(dump_path, "ab");
    if (!dump) {
      snprintf(err, errlen, "cannot open %s", dump_path);
      goto done;
    }
  }

  /* ---- time_integration_weak_coupling (CafeSolver.cpp:178-219) ---- */
  int32_t nb[26];
  {
    int c = 0;
    for (int k = -1; k < 2; k++)
      for (int j = -1; j < 2; j++)
        for (int i = -1; i < 2; i++) {
          if (k == 0 && j == 0 && i == 0) continue;
          nb[c++] = k * s->nxyg + j * s->nxg + i;
        }
  }
  struct timespec loop_t0, loop_t1;
  clock_gettime(CLOCK_MONOTONIC, &loop_t0);
  FE.dT = FE.ts0 - FE.ts1;   /* FiniteElementManager::setup_integration */
  double dT_FE = FE.dT;
  double maxTimestep = dT_FE; /* CellularAutomataManager::setup_integration */
  double time = 0.0, ca_time = 0.0, ca_dt = 0.0;
  int step = 0;
  int64_t tests = 0;
  int exhausted = 0;
  while (time < p->final_time && (max_steps < 0 || step < max_steps)) {
    /* checkup_current_temperature_to_update_phase_state (Remelting.cpp:339-404) */
    for (int64_t i = 0; i < N; ++i) {
      double T = nullMatTemp;
      int withMat = eval_temperature(&FE, R.tag, R.pc, i, void_t, &T);
      if (step > 0) {
        double rate = 410;
        if (R.T[i] > 0) rate = (T - R.T[i]) / ca_dt;
        if (T <= 0) rate = 0;
        R.cooling[i] = withMat ? (uint8_t)(rate < 0) : 0;
      }
      R.T[i] = T;
      if (is_ghost_cell(s, i)) continue;
      if (withMat && T < p->Tm) continue;
      s->orient[i] = -1;
      R.melted[i] = (uint8_t)(withMat ? 1 : 0);
    }
    /* checkup_liquid_cell_neigh_to_growth (Remelting.cpp:484-542) */
    memset(R.flag, 0, N);
    for (int i = 1; i < s->nxg - 1; i++)
      for (int j = 1; j < s->nyg - 1; j++)
        for (int k = 1; k < s->nzg - 1; k++) {
          int64_t c = (int64_t)k * s->nxyg + (int64_t)j * s->nxg + i;
          double T = R.T[c];
          int withMat = !(T < nullMatTemp + 0.01);
          if (s->orient[c] == -1 && withMat && time >= maxTimestep) R.melted[c] = 1;
          if (!withMat) {
            R.melted[c] = 0;
            continue;
          }
          if (s->orient[c] != -1) continue;
          if (T >= p->Tm) continue;
          for (int n = 0; n < 26; ++n)
            if (s->orient[c + nb[n]] > -1) R.flag[c + nb[n]] = 1;
        }
    /* calculate_time_step (Remelting.cpp:656-727) */
    if (p->nucleation) { /* nucleate_at_nucleation_sites (Remelting.cpp:936-999) */
      int64_t base = s->norient;
      int64_t local = 0;
      for (int64_t q = 0; q < s->nsites; ++q) {
        int32_t cell = s->sites[q];
        int isLiquid = (s->orient[cell] == -1);
        double T = R.T[cell];
        if (R.cooling[cell] && isLiquid && R.melted[cell] && T > p->Tnuc_min) {
          double dT = p->Tm - R.T[cell];
          if (dT > s->dtc[cell]) {
            int64_t o = remelt_new_orientation(s);
            if (o < 0) goto done;
            double c[3];
            cell_center(s, &R.g, cell, c);
            int32_t g = s->grain[cell];
            if (g == -1) {
              int64_t ng = remelt_new_grain(s, cell, (int32_t)o, c, 0.0);
              if (ng < 0) goto done;
              s->grain[cell] = (int32_t)ng;
            } else {
              s->len[g] = 0.0;
              s->xc[g] = c[0];
              s->yc[g] = c[1];
              s->zc[g] = c[2];
              s->gorient[g] = (int32_t)o;
            }
            s->orient[cell] = (int32_t)(base + local); /* update_global_orientation_list (:1205-1214) */
            local++;
          }
        }
      }
    }
    double minT = p->Tm;
    for (int i = 1; i < s->nxg - 1; i++)
      for (int j = 1; j < s->nyg - 1; j++)
        for (int k = 1; k < s->nzg - 1; k++) {
          int64_t c = (int64_t)k * s->nxyg + (int64_t)j * s->nxg + i;
          if (!R.flag[c]) continue;
          int32_t g = s->grain[c];
          if (g < 0) continue;
          double T = R.T[c];
          if (!(s->len[g] < cutoff)) s->len[g] = p->h;
          if (T <= p->Ts) continue;
          if (minT > T) minT = T;
        }
    double vmin = remelt_velocity(p, minT);
    double maxV = vmin > 0 ? vmin : 0;
    double a = p->time_step_factor_ca * p->h / maxV;
    double dtLoc = (maxTimestep < a) ? maxTimestep : a; /* std::min(a, maxTimestep_) */
    double dT = (dT_FE < dtLoc) ? dT_FE : dtLoc;        /* __min(dT_FE, dT_CA) */
    ca_dt = dT;
    FE.dT = dT;
    /* single_integration_step (Remelting.cpp:545-652): i-outer sweep, no cascade */
    for (int i = 1; i < s->nxg - 1; i++)
      for (int j = 1; j < s->nyg - 1; j++)
        for (int k = 1; k < s->nzg - 1; k++) {
          int64_t c = (int64_t)k * s->nxyg + (int64_t)j * s->nxg + i;
          if (!R.flag[c]) continue;
          int32_t g = s->grain[c];
          if (g < 0) continue;
          double T = R.T[c];
          double vel = (T < p->Ts) ? remelt_velocity(p, p->Ts + 0.01) : remelt_velocity(p, T);
          s->len[g] += dT * vel;
          const double *m = s->mat + 9 * (int64_t)s->gorient[g];
          for (int n = 0; n < 26; ++n) {
            int64_t nc = c + nb[n];
            double Tn = R.T[nc];
            if (s->orient[nc] > -1) continue;
            if (Tn > p->Tm) continue;
            if (!(Tn > nullMatTemp)) continue;
            if (is_ghost_cell(s, nc)) continue;
            if (s->len[g] == 0) continue; /* Octahedron::cell_is_captured: length 0 -> false */
            double cc[3], gc[3];
            cell_center(s, &R.g, nc, cc);
            gc[0] = cc[0] - s->xc[g];
            gc[1] = cc[1] - s->yc[g];
            gc[2] = cc[2] - s->zc[g];
            tests++;
            if (!amca_oracle_is_captured(m, gc, s->len[g])) continue;
            /* capture_cell (Remelting.cpp:807-847) */
            double info[4];
            double gcen[3] = {s->xc[g], s->yc[g], s->zc[g]};
            amca_oracle_capture(m, gc, s->len[g], p->h, p->trunc_coeff, info);
            double c3[3];
            for (int d = 0; d < 3; d++) c3[d] = info[d] + gcen[d];
            int32_t og = s->grain[nc];
            int32_t orient = s->gorient[g];
            if (og < 0) {
              int64_t ng = remelt_new_grain(s, (int32_t)nc, orient, c3, info[3]);
              if (ng < 0) goto done;
              s->grain[nc] = (int32_t)ng;
            } else {
              s->len[og] = info[3];
              s->xc[og] = c3[0];
              s->yc[og] = c3[1];
              s->zc[og] = c3[2];
              s->gorient[og] = orient;
            }
            s->orient[nc] = orient;
          }
        }
    ca_time += dT;
    step++;
    if (dump && remelt_dump(&R, &FE, dump, step == 1, step, ca_time, ca_dt, maxTimestep)) {
      snprintf(err, errlen, "dump write failed");
      goto done;
    }
    time += dT;
    int fr = fe_step(&FE, err, errlen);
    if (fr < 0) goto done;
    if (fr == 0) {
      exhausted = 1;
      break;
    }
    dT_FE = FE.ts0 - FE.time; /* get_max_time_step (LoadDataFromFile.cpp:197-205) */
    maxTimestep = dT_FE;
  }
  clock_gettime(CLOCK_MONOTONIC, &loop_t1);
  if (orient_out) memcpy(orient_out, s->orient, N * sizeof(int32_t));
  if (grain_out) memcpy(grain_out, s->grain, N * sizeof(int32_t));
  if (temp_out) memcpy(temp_out, R.T, N * sizeof(double));
  if (melted_out) memcpy(melted_out, R.melted, N);
  if (cooling_out) memcpy(cooling_out, R.cooling, N);
  if (flag_out) memcpy(flag_out, R.flag, N);
  if (res) {
    res->steps = step;
    res->time = time;
    res->last_dt = ca_dt;
    res->num_grains = s->ngrain;
    res->num_orient = s->norient;
    res->num_sites = s->nsites;
    res->tests = tests;
    res->nodes = FE.nnodes;
    res->elements = FE.nelem;
    res->frames_read = FE.frames;
    res->frames_exhausted = exhausted;
    res->loop_seconds = (double)(loop_t1.tv_sec - loop_t0.tv_sec) + 1e-9 * (double)(loop_t1.tv_nsec - loop_t0.tv_nsec);
  }
  rc = 0;
done:
  if (dump) fclose(dump);
  if (rc && !err[0]) snprintf(err, errlen, "out of memory");
  fe_free(&FE);
  remelt_free(&R);
  return rc;
}
