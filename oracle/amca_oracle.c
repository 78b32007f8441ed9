/*
 * amca_oracle.c — CPU restatement of AMCA3D's plain 3-D CA timestep.
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
#include "amca_oracle.h"

#include <math.h>
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
