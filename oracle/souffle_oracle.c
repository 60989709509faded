/* Oracle test infrastructure -- NOT the product.  See souffle_oracle.h.
 *
 * CPU restatement of SOUFFLE's force-and-integrate path.  Every function
 * names the reference lines it follows (paths relative to the
 * softmaterialslab/capsid-souffle tree).  Types mirror the reference:
 * VECTOR3D components are long double (src/vector3d.h:22), bead/edge/face
 * scalars are double (src/bead.h:28-51, src/edge.h:21-22, src/face.h:21-22),
 * so with ORACLE_REAL = long double on x86-64 the results match the compiled
 * reference exactly.
 */
#include "souffle_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL long double
#endif
typedef ORACLE_REAL real;

#define SQRT(x) _Generic((x), long double: sqrtl, default: sqrt)(x)
#define EXP(x) _Generic((x), long double: expl, default: exp)(x)
#define POW(x, y) _Generic((x), long double: powl, default: pow)(x, y)

typedef struct { real x, y, z; } vec3;

static inline vec3 v3(real x, real y, real z) { vec3 r = {x, y, z}; return r; }
static inline vec3 vsub(vec3 a, vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3 vadd(vec3 a, vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline real vdot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* operator& of src/vector3d.h:343-345 */
static inline vec3 vcross(vec3 a, vec3 b) {
  return v3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
/* operator^ of src/vector3d.h:346-348: the scalar is a long double */
static inline vec3 vscale(vec3 a, real s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline real vnorm2(vec3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
/* VECTOR3D::GetMagnitude (src/vector3d.h:31-33) calls unqualified sqrt in a
 * header without `using namespace std`, which binds to C's double sqrt(double):
 * the long double sum is rounded to double, rooted in double, and widened back.
 * Edge lengths, face areas, energy distances and kinetic energies all go
 * through it.  The pair loop's sqrt(r2) (src/forces.cpp:101) sits after
 * `using namespace std` and is a true long double root. */
static inline real vnorm(vec3 a) { return (real)sqrt((double)(a.x * a.x + a.y * a.y + a.z * a.z)); }

/* Single-shift minimum image used at every call site, e.g. src/functions.h:42-56. */
static inline vec3 pbc(vec3 r, real bx, real hbx) {
  if (r.x > hbx) r.x -= bx;
  else if (r.x < -hbx) r.x += bx;
  if (r.y > hbx) r.y -= bx;
  else if (r.y < -hbx) r.y += bx;
  if (r.z > hbx) r.z -= bx;
  else if (r.z < -hbx) r.z += bx;
  return r;
}

struct oracle_sys {
  oracle_desc d;
  int n;               /* beads */
  /* copies of the template */
  int *b_type, *e_b, *e_type, *f_b, *lj_t;
  double *b_q, *b_sigma, *b_mass, *e_len0;
  /* derived template topology */
  int *e_f;            /* [ne*2] faces of each edge, face order (-1 if absent) */
  int *bead_edges;     /* [np*maxdeg] edges of each bead in template edge order */
  int *bead_nedge;     /* [np] */
  int maxdeg;
  /* state (reference types) */
  vec3 *pos, *vel, *tforce, *sforce, *bforce;
  double *ke;          /* BEAD::ke */
  double *se, *be, *ne, *ce;
  double *e_length;    /* EDGE::length, per global edge */
  vec3 *e_lvec;        /* EDGE::lengthvec */
  vec3 *f_nrm, *f_area; /* FACE::normvec / areavector */
  double *f_a;         /* FACE::a */
  int *nl;             /* [n*cap] BEAD::itsN, -1 padded */
  int *nl_count;
  int overflow;
  real bx, hbx;
  /* encapsulation big beads (static): positions, diameter, charge, hard-core distance, and the
     big-bead sums of the last energy block (src/md.cpp:606-614) */
  int nbb;
  vec3* bb_pos;
  double bb_sigma, bb_q, bb_shc;
  double bb_ne_tot, bb_ce_tot;
};

static int threads_req = 0;
void oracle_set_threads(int n) { threads_req = n; }

int oracle_center_bead(int np, const double* pos, double box) {
  /* src/initialize.cpp:266-288 */
  vec3 c = v3(0, 0, 0);
  for (int i = 0; i < np; i++) c = vadd(c, v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
  c = v3(c.x / (real)np, c.y / (real)np, c.z / (real)np);
  real old = 1000, bx = (real)box, hbx = bx / 2;
  int id = 0;
  for (int i = 0; i < np; i++) {
    vec3 r = vsub(v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), c);
    r = pbc(r, bx, hbx);
    real d = vnorm2(r);
    if (d < old) {
      old = d;
      id = i;
    }
  }
  return id;
}

#define DUP(dst, src, cnt, T)                              \
  do {                                                     \
    dst = (T*)malloc(sizeof(T) * ((cnt) > 0 ? (cnt) : 1)); \
    if ((cnt) > 0) memcpy(dst, src, sizeof(T) * (cnt));    \
  } while (0)

oracle_sys* oracle_create(const oracle_desc* d) {
  oracle_sys* s = (oracle_sys*)calloc(1, sizeof(oracle_sys));
  s->d = *d;
  const int np = d->np, ne = d->ne, nf = d->nf;
  s->n = d->n_sub * np;
  DUP(s->b_type, d->b_type, np, int);
  DUP(s->b_q, d->b_q, np, double);
  DUP(s->b_sigma, d->b_sigma, np, double);
  DUP(s->b_mass, d->b_mass, np, double);
  DUP(s->e_b, d->e_b, 2 * ne, int);
  DUP(s->e_type, d->e_type, ne, int);
  DUP(s->e_len0, d->e_len0, ne, double);
  DUP(s->f_b, d->f_b, 3 * nf, int);
  DUP(s->lj_t, d->lj_t, 2 * d->n_lj, int);

  /* Face <-> edge matching (src/initialize.cpp:370-401): faces are appended to
   * an edge's itsF in face order; a face matches an edge on any of its three
   * sides, in either orientation. */
  s->e_f = (int*)malloc(sizeof(int) * 2 * (ne > 0 ? ne : 1));
  int* nfe = (int*)calloc(ne > 0 ? ne : 1, sizeof(int));
  for (int k = 0; k < 2 * ne; k++) s->e_f[k] = -1;
  for (int f = 0; f < nf; f++) {
    const int a = s->f_b[3 * f], b = s->f_b[3 * f + 1], c = s->f_b[3 * f + 2];
    for (int e = 0; e < ne; e++) {
      const int e0 = s->e_b[2 * e], e1 = s->e_b[2 * e + 1];
      int hits = 0;
      if (a == e0 && b == e1) hits++;
      else if (a == e1 && b == e0) hits++;
      if (a == e0 && c == e1) hits++;
      else if (a == e1 && c == e0) hits++;
      if (b == e1 && c == e0) hits++;
      else if (b == e0 && c == e1) hits++;
      for (int h = 0; h < hits; h++) {
        if (nfe[e] < 2) s->e_f[2 * e + nfe[e]] = f;
        nfe[e]++;
      }
    }
  }
  for (int e = 0; e < ne; e++) {
    if (s->e_type[e] != 0 && nfe[e] < 2) {
      free(nfe);
      oracle_destroy(s);
      return NULL;
    }
  }
  free(nfe);

  /* BEAD::itsE in template edge order (src/initialize.cpp:328-329). */
  s->bead_nedge = (int*)calloc(np, sizeof(int));
  for (int e = 0; e < ne; e++) {
    s->bead_nedge[s->e_b[2 * e]]++;
    s->bead_nedge[s->e_b[2 * e + 1]]++;
  }
  s->maxdeg = 1;
  for (int i = 0; i < np; i++)
    if (s->bead_nedge[i] > s->maxdeg) s->maxdeg = s->bead_nedge[i];
  s->bead_edges = (int*)malloc(sizeof(int) * np * s->maxdeg);
  memset(s->bead_nedge, 0, sizeof(int) * np);
  for (int e = 0; e < ne; e++) {
    int b0 = s->e_b[2 * e], b1 = s->e_b[2 * e + 1];
    s->bead_edges[b0 * s->maxdeg + s->bead_nedge[b0]++] = e;
    s->bead_edges[b1 * s->maxdeg + s->bead_nedge[b1]++] = e;
  }

  const int n = s->n;
  s->pos = (vec3*)calloc(n, sizeof(vec3));
  s->vel = (vec3*)calloc(n, sizeof(vec3));
  s->tforce = (vec3*)calloc(n, sizeof(vec3));
  s->sforce = (vec3*)calloc(n, sizeof(vec3));
  s->bforce = (vec3*)calloc(n, sizeof(vec3));
  s->ke = (double*)calloc(n, sizeof(double));
  s->se = (double*)calloc(n, sizeof(double));
  s->be = (double*)calloc(n, sizeof(double));
  s->ne = (double*)calloc(n, sizeof(double));
  s->ce = (double*)calloc(n, sizeof(double));
  s->e_length = (double*)calloc((size_t)d->n_sub * ne + 1, sizeof(double));
  s->e_lvec = (vec3*)calloc((size_t)d->n_sub * ne + 1, sizeof(vec3));
  s->f_nrm = (vec3*)calloc((size_t)d->n_sub * nf + 1, sizeof(vec3));
  s->f_area = (vec3*)calloc((size_t)d->n_sub * nf + 1, sizeof(vec3));
  s->f_a = (double*)calloc((size_t)d->n_sub * nf + 1, sizeof(double));
  s->nl = (int*)malloc(sizeof(int) * (size_t)n * d->nlist_capacity);
  for (size_t k = 0; k < (size_t)n * d->nlist_capacity; k++) s->nl[k] = -1;
  s->nl_count = (int*)calloc(n, sizeof(int));
  /* box: a double value held in long double (src/initialize.cpp:49-51) */
  s->bx = (real)d->box;
  s->hbx = s->bx * (real)0.5;
  return s;
}

void oracle_destroy(oracle_sys* s) {
  if (!s) return;
  void* ptrs[] = {s->b_type, s->e_b,     s->e_type, s->f_b,    s->lj_t,     s->b_q,
                  s->b_sigma, s->b_mass, s->e_len0, s->e_f,    s->bead_edges, s->bead_nedge,
                  s->pos,    s->vel,     s->tforce, s->sforce, s->bforce,   s->ke,
                  s->se,     s->be,      s->ne,     s->ce,     s->e_length, s->e_lvec,
                  s->f_nrm,  s->f_area,  s->f_a,    s->nl,     s->nl_count, s->bb_pos};
  for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) free(ptrs[k]);
  free(s);
}

void oracle_set_state(oracle_sys* s, const double* pos, const double* vel) {
  for (int i = 0; i < s->n; i++) {
    /* positions are parsed into long double (src/initialize.cpp:74,214),
       velocities into double (src/initialize.cpp:196,214) */
    s->pos[i] = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    if (vel) s->vel[i] = v3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
  }
}

void oracle_get_state(const oracle_sys* s, double* pos, double* vel) {
  for (int i = 0; i < s->n; i++) {
    if (pos) {
      pos[3 * i] = (double)s->pos[i].x;
      pos[3 * i + 1] = (double)s->pos[i].y;
      pos[3 * i + 2] = (double)s->pos[i].z;
    }
    if (vel) {
      vel[3 * i] = (double)s->vel[i].x;
      vel[3 * i + 1] = (double)s->vel[i].y;
      vel[3 * i + 2] = (double)s->vel[i].z;
    }
  }
}

/* ---------------------------------------------------------------------------
 * update_pairlist (src/functions.cpp:69-117) for subunit i.  Reproduces the
 * centre-bead prefilter (1.5 x cutoff on centre-bead distance, :80-91) and the
 * stale-r2 reuse for pairs touching subunit 0's centre bead: the test at :97
 * compares a local bead index with a global bead id, so only subunit 0's
 * centre bead ever matches.  Returns the number of entries that did not fit. */
static int pairlist_subunit(oracle_sys* s, int i) {
  const int np = s->d.np, S = s->d.n_sub, cap = s->d.nlist_capacity;
  const double nl2 = s->d.nlist_cutoff * s->d.nlist_cutoff;
  const int cid_i = i * np + s->d.center_local; /* centerBead->id: a global id */
  real r2 = 0.0;
  int over = 0;
  for (int ii = 0; ii < np; ii++) {
    int g = i * np + ii;
    for (int k = 0; k < cap; k++) s->nl[(size_t)g * cap + k] = -1;
    s->nl_count[g] = 0;
  }
  for (int j = 0; j < S; j++) {
    const int cid_j = j * np + s->d.center_local;
    if (i != j) {
      vec3 r = vsub(s->pos[cid_i], s->pos[cid_j]);
      r = pbc(r, s->bx, s->hbx);
      r2 = vnorm2(r);
    } else {
      r2 = 0;
    }
    if (r2 < (nl2 * 2.25)) {
      for (int ii = 0; ii < np; ii++) {
        const int gi = i * np + ii;
        for (int jj = 0; jj < np; jj++) {
          const int gj = j * np + jj;
          const int electrostatic = (gi != gj && s->b_q[ii] != 0 && s->b_q[jj] != 0);
          const int lj = (i != j);
          if (electrostatic || lj) {
            if (ii != cid_i && jj != cid_j) {
              vec3 r = vsub(s->pos[gi], s->pos[gj]);
              r = pbc(r, s->bx, s->hbx);
              r2 = vnorm2(r);
            }
            if (r2 < nl2) {
              int c = s->nl_count[gi];
              if (c < cap) s->nl[(size_t)gi * cap + c] = gj;
              else over++;
              s->nl_count[gi] = c + 1;
            }
          }
        }
      }
    }
  }
  return over;
}

/* FACE::across (src/face.cpp:27-34) */
static inline int face_across(const oracle_sys* s, int fglob_base, int f, int b0, int b1) {
  for (int k = 0; k < 3; k++) {
    int b = fglob_base + s->f_b[3 * f + k];
    if (b != b0 && b != b1) return b;
  }
  return -1;
}

/* EDGE::get_gradS (src/edge.cpp:98-161) */
static vec3 grad_s(int wrt, int b0, int b1, int fb0, int fb1, const int* f0b, const int* f1b,
                   vec3 r13, vec3 r01, vec3 r12, vec3 r02, vec3 r03) {
  (void)fb0;
  (void)fb1;
  vec3 result = v3(0, 0, 0);
  if (wrt == b0 || wrt == b1) {
    vec3 d23, d32, d20, d21;
    if (wrt == b0) {
      d23 = r13;
      d32 = vscale(r13, -1);
      d20 = vscale(r01, -1);
      d21 = r12;
    } else {
      d23 = r03;
      d32 = vscale(r03, -1);
      d20 = r01;
      d21 = r02;
    }
    vec3 c2021 = vcross(d20, d21), c2032 = vcross(d20, d32);
    result.x = d23.y * c2021.z - d21.y * c2032.z + d32.z * c2021.y + d21.z * c2032.y;
    result.y = d32.x * c2021.z + d21.x * c2032.z + d23.z * c2021.x - d21.z * c2032.x;
    result.z = d23.x * c2021.y - d21.x * c2032.y + d32.y * c2021.x + d21.y * c2032.x;
  } else {
    vec3 r1x = v3(0, 0, 0);
    for (int k = 0; k < 3; k++)
      if (f0b[k] != b0 && f0b[k] != b1 && f0b[k] != wrt) r1x = vscale(r12, -1);
    for (int k = 0; k < 3; k++)
      if (f1b[k] != b0 && f1b[k] != b1 && f1b[k] != wrt) r1x = vscale(r13, -1);
    result = vcross(r01, vcross(r01, r1x));
  }
  return result;
}

/* Forces for one subunit: src/forces.cpp:36-145 with the member functions it
 * calls (src/edge.cpp:35-49,69-96,163-188; src/face.cpp:11-17;
 * src/bead.cpp:17-23). */
static void forces_subunit(oracle_sys* s, int i) {
  const int np = s->d.np, ne = s->d.ne, nf = s->d.nf;
  const int base = i * np;
  const double ks = s->d.ks, kb = s->d.kb;
  const real bx = s->bx, hbx = s->hbx;

  for (int e = 0; e < ne; e++) { /* EDGE::update_length */
    const int ge = i * ne + e;
    vec3 lv = vsub(s->pos[base + s->e_b[2 * e]], s->pos[base + s->e_b[2 * e + 1]]);
    const real half = bx * (real)0.5;
    lv = pbc(lv, bx, half);
    s->e_lvec[ge] = lv;
    s->e_length[ge] = (double)vnorm(lv);
  }
  for (int f = 0; f < nf; f++) { /* FACE::update_area_normal */
    const int gf = i * nf + f;
    const int a = base + s->f_b[3 * f], b = base + s->f_b[3 * f + 1], c = base + s->f_b[3 * f + 2];
    vec3 first = pbc(vsub(s->pos[b], s->pos[a]), bx, hbx);
    vec3 second = pbc(vsub(s->pos[c], s->pos[b]), bx, hbx);
    vec3 av = vscale(vcross(first, second), (real)0.5);
    s->f_area[gf] = av;
    s->f_a[gf] = (double)vnorm(av);
    s->f_nrm[gf] = vscale(av, (real)(1 / s->f_a[gf]));
  }
  for (int ii = 0; ii < np; ii++) { /* BEAD::update_stretching_force */
    const int g = base + ii;
    vec3 sf = v3(0, 0, 0);
    for (int k = 0; k < s->bead_nedge[ii]; k++) {
      const int e = s->bead_edges[ii * s->maxdeg + k];
      const int other = base + (s->e_b[2 * e] == ii ? s->e_b[2 * e + 1] : s->e_b[2 * e]);
      vec3 r = pbc(vsub(s->pos[g], s->pos[other]), bx, hbx);
      const double len = s->e_length[i * ne + e];
      sf = vadd(sf, vscale(r, (real)((s->e_len0[e] - len) * ks / len)));
    }
    s->sforce[g] = sf;
    s->bforce[g] = v3(0, 0, 0);
  }
  for (int e = 0; e < ne; e++) { /* EDGE::update_bending_forces */
    if (s->e_type[e] == 0) continue;
    const int f0 = s->e_f[2 * e], f1 = s->e_f[2 * e + 1];
    const int gf0 = i * nf + f0, gf1 = i * nf + f1;
    const int b0 = base + s->e_b[2 * e], b1 = base + s->e_b[2 * e + 1];
    const int r2b = face_across(s, base, f0, b0, b1);
    const int r3b = face_across(s, base, f1, b0, b1);
    if (vdot(s->f_nrm[gf0], s->f_nrm[gf1]) < 0) { /* in-place flip, src/edge.cpp:78-81 */
      s->f_nrm[gf1] = vscale(s->f_nrm[gf1], -1);
      s->f_area[gf1] = vscale(s->f_area[gf1], -1);
    }
    const double S = (double)(vdot(s->f_area[gf0], s->f_area[gf1]) * 4);
    const double a0 = s->f_a[gf0], a1 = s->f_a[gf1];
    const vec3 d01 = s->e_lvec[i * ne + e];
    const vec3 d02 = pbc(vsub(s->pos[b0], s->pos[r2b]), bx, hbx);
    const vec3 d03 = pbc(vsub(s->pos[b0], s->pos[r3b]), bx, hbx);
    const vec3 d12 = pbc(vsub(s->pos[b1], s->pos[r2b]), bx, hbx);
    const vec3 d13 = pbc(vsub(s->pos[b1], s->pos[r3b]), bx, hbx);
    int f0b[3], f1b[3];
    for (int k = 0; k < 3; k++) {
      f0b[k] = base + s->f_b[3 * f0 + k];
      f1b[k] = base + s->f_b[3 * f1 + k];
    }
    const int rr[4] = {b0, b1, r2b, r3b};
    for (int q = 0; q < 4; q++) {
      const int w = rr[q];
      vec3 gs = grad_s(w, b0, b1, f0, f1, f0b, f1b, d13, d01, d12, d02, d03);
      vec3 g0 = v3(0, 0, 0), g1 = v3(0, 0, 0);
      if (w == b0) g0 = vscale(vcross(d12, vcross(d02, d01)), -1);
      else if (w == b1) g0 = vcross(d02, vcross(d12, d01));
      else if (w == r2b) g0 = vscale(vcross(d01, vcross(d02, d01)), -1);
      else if (w == r3b) g0 = v3(0, 0, 0);
      g0 = vscale(g0, (real)(0.25 / a0));
      if (w == b0) g1 = vscale(vcross(d13, vcross(d03, d01)), -1);
      else if (w == b1) g1 = vcross(d03, vcross(d13, d01));
      else if (w == r3b) g1 = vscale(vcross(d01, vcross(d03, d01)), -1);
      else if (w == r2b) g1 = v3(0, 0, 0);
      g1 = vscale(g1, (real)(0.25 / a1));
      vec3 t = vsub(gs, vadd(vscale(g0, (real)(S / a0)), vscale(g1, (real)(S / a1))));
      s->bforce[w] = vadd(s->bforce[w], vscale(t, (real)(kb / (a0 * a1 * 4))));
    }
  }
}

/* Pair loop for one subunit: src/forces.cpp:67-145. */
static void pairs_subunit(oracle_sys* s, int i) {
  const int np = s->d.np, cap = s->d.nlist_capacity;
  const double ecut_el2 = s->d.ecut_el * s->d.ecut_el;
  const double ecut2 = s->d.ecut * s->d.ecut;
  const double replj2 = 1.12246205 * 1.12246205;
  const double kappa = s->d.kappa, lb = s->d.lb, ecut_el = s->d.ecut_el;
  const real bx = s->bx, hbx = s->hbx;
  real r2 = 0.0;
  vec3 r_vec = v3(0, 0, 0);
  for (int ii = 0; ii < np; ii++) {
    const int gi = i * np + ii;
    vec3 eF = v3(0, 0, 0), ljF = v3(0, 0, 0);
    for (int jj = 0; jj < cap; jj++) {
      const int gj = s->nl[(size_t)gi * cap + jj];
      if (gj == -1) break;
      const int lj_j = gj % np, sub_j = gj / np;
      const double qi = s->b_q[ii], qj = s->b_q[lj_j];
      const int electrostatic = (gi != gj && qi != 0 && qj != 0);
      const int lj = (i != sub_j);
      real r = 0.0;
      if (electrostatic || lj) {
        r_vec = pbc(vsub(s->pos[gi], s->pos[gj]), bx, hbx);
        r2 = vnorm2(r_vec);
      }
      const double sig1 = s->b_sigma[ii], sig2 = s->b_sigma[lj_j];
      const double shc = (sig1 + sig2) / 2;
      const double yukawa_scale = exp(kappa * shc) / ((1 + kappa * sig1 / 2) * (1 + kappa * sig2 / 2));
      if ((electrostatic && r2 < ecut_el2 && ecut_el != 0) || (electrostatic && ecut_el == 0)) {
        r = SQRT(r2);
        eF = vadd(eF, vscale(r_vec, ((qi * qj * lb * EXP(-kappa * r) / (r2)) * (kappa + 1 / r) *
                                     yukawa_scale)));
      }
      if (r2 >= ecut2 && r2 >= (replj2 * shc * shc)) continue;
      if (lj) {
        int att = 0;
        for (int k = 0; k < s->d.n_lj; k++) {
          if (s->b_type[ii] == s->lj_t[2 * k] && s->b_type[lj_j] == s->lj_t[2 * k + 1]) {
            att = 1;
            break;
          }
        }
        if (att && r2 < ecut2) {
          const double test = (s->b_type[lj_j] == 7) ? 50 : s->d.elj_att;
          const double r6 = (double)(r2 * r2 * r2);
          const double sigma6 = sig1 * sig1 * sig1 * sig1 * sig1 * sig1;
          ljF = vadd(ljF, vscale(r_vec, (48 * test * ((sigma6 / r6) * ((sigma6 / r6) - 0.5))) *
                                            (1 / (r2))));
        } else if (!att && r2 < (replj2 * shc * shc)) {
          const double r6 = (double)(r2 * r2 * r2);
          const double sigma6 = shc * shc * shc * shc * shc * shc;
          const double elj = 1;
          ljF = vadd(ljF, vscale(r_vec, (48 * elj * ((sigma6 / r6) * ((sigma6 / r6) - 0.5))) *
                                            (1 / (r2))));
        }
      }
    }
    s->tforce[gi] = vadd(vadd(s->sforce[gi], s->bforce[gi]), vadd(eF, ljF));
  }
}

void oracle_set_big_beads(oracle_sys* s, int n, const double* pos, double sigma, double charge, double shc) {
  free(s->bb_pos);
  s->bb_pos = NULL;
  s->nbb = n > 0 ? n : 0;
  if (s->nbb) s->bb_pos = (vec3*)malloc(sizeof(vec3) * (size_t)n);
  /* restart positions are read into the long double vector (src/initialize.cpp:584-587) */
  for (int i = 0; i < s->nbb; i++) s->bb_pos[i] = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  s->bb_sigma = sigma;
  s->bb_q = charge;
  s->bb_shc = shc;
  s->bb_ne_tot = s->bb_ce_tot = 0;
}

/* forceCalculation_bigbead (src/forces.cpp:174-236): every big bead with every subunit bead;
 * the subunit bead's eforce / ljforce start at zero, take minus each pair force in big-bead
 * order, and join tforce as tforce + ljforce + eforce.  r is GetMagnitude (a double root),
 * r2 the long double square; pow(r - delta, 6) is a long double power rounded to double. */
static void bigbead_forces(oracle_sys* s) {
  const int n = s->n, np = s->d.np;
  const real bx = s->bx, hbx = s->hbx;
  const double ecut_el = s->d.ecut_el, kappa = s->d.kappa, lb = s->d.lb, shc = s->bb_shc;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < n; j++) {
    vec3 ef = v3(0, 0, 0), lf = v3(0, 0, 0);
    const double qj = s->b_q[j % np];
    const int electrostatic = (qj != 0);
    for (int i = 0; i < s->nbb; i++) {
      vec3 eForce = v3(0, 0, 0), ljForce = v3(0, 0, 0);
      const vec3 r_vec = pbc(vsub(s->bb_pos[i], s->pos[j]), bx, hbx);
      const real r = vnorm(r_vec);
      const real r2 = vnorm2(r_vec);
      const double sig1 = s->bb_sigma, sig2 = s->b_sigma[j % np];
      const double sigavg = (sig1 + sig2) / 2;
      const double delta = sigavg - shc;
      const double shc6 = pow(shc, 6);
      const double r6 = (double)POW(r - delta, (real)6);
      const double yukawa_scale = exp(kappa * sigavg) / ((1 + kappa * sig1 / 2) * (1 + kappa * sig2 / 2));
      if (electrostatic && r2 < (ecut_el * ecut_el))
        eForce = vscale(r_vec, ((s->bb_q * qj * lb * EXP(-kappa * r) / (r2)) * (kappa + 1 / r) * yukawa_scale));
      if (r2 < (delta + 1.12246205 * shc) * (delta + 1.12246205 * shc))
        ljForce = vscale(r_vec, (48 * ((shc6 / r6) * ((shc6 / r6) - 0.5))) * (1 / r) * (1 / (r - delta)));
      ef = vsub(ef, eForce);
      lf = vsub(lf, ljForce);
    }
    s->tforce[j] = vadd(vadd(s->tforce[j], lf), ef);
  }
}

void oracle_big_bead_energies(const oracle_sys* s, double* big_ne, double* big_ce) {
  if (big_ne) *big_ne = s->bb_ne_tot;
  if (big_ce) *big_ce = s->bb_ce_tot;
}

int oracle_forces(oracle_sys* s, int rebuild) {
  const int S = s->d.n_sub;
  int over = 0;
#ifdef _OPENMP
  if (threads_req > 0) omp_set_num_threads(threads_req);
#endif
  /* src/forces.cpp:33-146: dynamic schedule over subunits */
#pragma omp parallel for schedule(dynamic) reduction(+ : over)
  for (int i = 0; i < S; i++) {
    forces_subunit(s, i);
    if (rebuild) over += pairlist_subunit(s, i);
    pairs_subunit(s, i);
  }
  s->overflow = over;
  if (s->nbb > 0) bigbead_forces(s);
  return over;
}

void oracle_get_forces(const oracle_sys* s, double* tf, double* sf, double* bf) {
  for (int i = 0; i < s->n; i++) {
    if (tf) {
      tf[3 * i] = (double)s->tforce[i].x;
      tf[3 * i + 1] = (double)s->tforce[i].y;
      tf[3 * i + 2] = (double)s->tforce[i].z;
    }
    if (sf) {
      sf[3 * i] = (double)s->sforce[i].x;
      sf[3 * i + 1] = (double)s->sforce[i].y;
      sf[3 * i + 2] = (double)s->sforce[i].z;
    }
    if (bf) {
      bf[3 * i] = (double)s->bforce[i].x;
      bf[3 * i + 1] = (double)s->bforce[i].y;
      bf[3 * i + 2] = (double)s->bforce[i].z;
    }
  }
}

void oracle_get_pairlist(const oracle_sys* s, int* counts, int* ids) {
  const int cap = s->d.nlist_capacity;
  for (int i = 0; i < s->n; i++) {
    if (counts) counts[i] = s->nl_count[i];
    if (ids) memcpy(ids + (size_t)i * cap, s->nl + (size_t)i * cap, sizeof(int) * cap);
  }
}

/* BEAD::update_kinetic_energy (src/bead.h:129-131) + particle_kinetic_energy
 * (src/energies.cpp:13-22) */
double oracle_kinetic_energy(oracle_sys* s) {
  for (int i = 0; i < s->n; i++) {
    const double m = s->b_mass[i % s->d.np];
    s->ke[i] = (double)(0.5 * m * vnorm(s->vel[i]) * vnorm(s->vel[i]));
  }
  real k = 0.0;
  for (int i = 0; i < s->n; i++) k += s->ke[i];
  return (double)k;
}

static real kinetic_energy_real(oracle_sys* s) {
  for (int i = 0; i < s->n; i++) {
    const double m = s->b_mass[i % s->d.np];
    s->ke[i] = (double)(0.5 * m * vnorm(s->vel[i]) * vnorm(s->vel[i]));
  }
  real k = 0.0;
  for (int i = 0; i < s->n; i++) k += s->ke[i];
  return k;
}

/* Energy block of src/md.cpp:553-583. */
void oracle_energies(oracle_sys* s, double* se, double* ke, double* be, double* neo, double* ce) {
  const int np = s->d.np, ne = s->d.ne, nf = s->d.nf, S = s->d.n_sub, n = s->n;
  const real bx = s->bx, hbx = s->hbx;
  /* dress_up (src/functions.cpp:60-67) */
  for (int i = 0; i < S; i++) {
    const int base = i * np;
    for (int e = 0; e < ne; e++) {
      vec3 lv = vsub(s->pos[base + s->e_b[2 * e]], s->pos[base + s->e_b[2 * e + 1]]);
      lv = pbc(lv, bx, bx * (real)0.5);
      s->e_lvec[i * ne + e] = lv;
      s->e_length[i * ne + e] = (double)vnorm(lv);
    }
    for (int f = 0; f < nf; f++) {
      const int gf = i * nf + f;
      const int a = base + s->f_b[3 * f], b = base + s->f_b[3 * f + 1], c = base + s->f_b[3 * f + 2];
      vec3 first = pbc(vsub(s->pos[b], s->pos[a]), bx, hbx);
      vec3 second = pbc(vsub(s->pos[c], s->pos[b]), bx, hbx);
      vec3 av = vscale(vcross(first, second), (real)0.5);
      s->f_area[gf] = av;
      s->f_a[gf] = (double)vnorm(av);
      s->f_nrm[gf] = vscale(av, (real)(1 / s->f_a[gf]));
    }
  }
  for (int g = 0; g < n; g++) s->be[g] = s->ne[g] = s->ce[g] = 0;
  for (int i = 0; i < S; i++) {
    const int base = i * np;
    for (int ii = 0; ii < np; ii++) {
      /* BEAD::update_stretching_energy (src/bead.cpp:9-14) */
      double acc = 0;
      for (int k = 0; k < s->bead_nedge[ii]; k++) {
        const int e = s->bead_edges[ii * s->maxdeg + k];
        const double dl = s->e_len0[e] - s->e_length[i * ne + e];
        acc += (0.25 * s->d.ks * dl * dl);
      }
      s->se[base + ii] = acc;
      const double m = s->b_mass[ii];
      s->ke[base + ii] = (double)(0.5 * m * vnorm(s->vel[base + ii]) * vnorm(s->vel[base + ii]));
    }
    for (int e = 0; e < ne; e++) { /* EDGE::update_bending_energy (src/edge.cpp:51-67) */
      if (s->e_type[e] == 0) continue;
      const int f0 = s->e_f[2 * e], f1 = s->e_f[2 * e + 1];
      const int gf0 = i * nf + f0, gf1 = i * nf + f1;
      const int b0 = base + s->e_b[2 * e], b1 = base + s->e_b[2 * e + 1];
      const int rr[4] = {b0, b1, face_across(s, base, f0, b0, b1), face_across(s, base, f1, b0, b1)};
      if (vdot(s->f_nrm[gf0], s->f_nrm[gf1]) < 0) {
        s->f_nrm[gf1] = vscale(s->f_nrm[gf1], -1);
        s->f_area[gf1] = vscale(s->f_area[gf1], -1);
      }
      for (int q = 0; q < 4; q++) /* double += long double: summed in long double */
        s->be[rr[q]] = (double)(s->be[rr[q]] +
                                s->d.kb * 0.25 * (1 - vdot(s->f_nrm[gf0], s->f_nrm[gf1])));
    }
  }
  /* update_LJ_ES_energies_simplified (src/energies.cpp:24-93): all pairs j > i */
  const double ecut = s->d.ecut, ecut_el = s->d.ecut_el, kappa = s->d.kappa, lb = s->d.lb;
  const double ecut3 = ecut * ecut * ecut, ecut6 = ecut3 * ecut3;
  /* Speed only, results unchanged: a pair whose minimum-image distance (in double, with a
   * 1e-6 relative margin) lies beyond the DH cut-off, the LJ cut-off and the WCA range of the
   * widest bead pair adds exactly nothing below, so it is skipped before the long double
   * arithmetic.  With no DH cut-off (ecut_el == 0) every pair is evaluated. */
  double sig_max = 0;
  for (int l = 0; l < np; l++) sig_max = s->b_sigma[l] > sig_max ? s->b_sigma[l] : sig_max;
  double reach = ecut_el > ecut ? ecut_el : ecut;
  if (1.12246205 * sig_max > reach) reach = 1.12246205 * sig_max;
  reach *= 1.000001;
  const double reach2 = reach * reach, box_d = (double)bx;
  const int prefilter = (ecut_el != 0);
  double* pd = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  for (int g = 0; g < n; g++) {
    pd[3 * g] = (double)s->pos[g].x;
    pd[3 * g + 1] = (double)s->pos[g].y;
    pd[3 * g + 2] = (double)s->pos[g].z;
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; i++) {
    const int li = i % np, si = i / np;
    for (int j = i + 1; j < n; j++) {
      if (prefilter) {
        double r2 = 0;
        for (int a = 0; a < 3; a++) {
          double dd = fabs(pd[3 * i + a] - pd[3 * j + a]);
          if (dd > box_d - dd) dd = box_d - dd;
          r2 += dd * dd;
        }
        if (r2 > reach2) continue;
      }
      const int lj_ = j % np, sj = j / np;
      const double qi = s->b_q[li], qj = s->b_q[lj_];
      const int electrostatic = (i != j && qi != 0 && qj != 0);
      const int lj = (si != sj);
      real r = 0.0;
      if (electrostatic || lj) r = vnorm(pbc(vsub(s->pos[i], s->pos[j]), bx, hbx));
      const double sig1 = s->b_sigma[li], sig2 = s->b_sigma[lj_];
      const double shc = (sig1 + sig2) / 2;
      const double ys = exp(kappa * shc) / ((1 + kappa * sig1 / 2) * (1 + kappa * sig2 / 2));
      if (electrostatic && r < ecut_el && ecut_el != 0) {
        s->ce[i] = (double)(s->ce[i] + ys * ((qi * qj * lb * EXP(-kappa * r)) / (r) -
                                             ((qi * qj * lb * exp(-kappa * ecut_el)) / (ecut_el))));
      } else if (electrostatic && ecut_el == 0) {
        s->ce[i] = (double)(s->ce[i] + (qi * qj * lb * EXP(-kappa * r) * ys) / (r));
      } else {
        s->ce[i] += 0;
      }
      const double sigma3 = shc * shc * shc, sigma6 = sigma3 * sigma3;
      const double r3 = (double)(r * r * r), r6 = r3 * r3;
      if (r >= ecut && r >= (1.12246205 * shc)) continue;
      if (lj) {
        int att = 0;
        for (int k = 0; k < s->d.n_lj; k++)
          if (s->b_type[li] == s->lj_t[2 * k] && s->b_type[lj_] == s->lj_t[2 * k + 1]) {
            att = 1;
            break;
          }
        if (r < (1.12246205 * shc) && !att) {
          const double elj = 1;
          s->ne[i] += ((4 * elj * (sigma6 / r6) * ((sigma6 / r6) - 1)) + elj);
        } else if (r < ecut && att) {
          s->ne[i] += (((4 * s->d.elj_att * (sigma6 / r6) * ((sigma6 / r6) - 1)) -
                        (4 * s->d.elj_att * ((sigma6 / ecut6) * ((sigma6 / ecut6) - 1)))));
        } else {
          s->ne[i] += 0;
        }
      }
    }
  }
  free(pd);
  if (s->nbb > 0) {
    /* update_LJ_ES_energies_bigbeads (src/energies.cpp:96-137): credited to both beads; the
       big-bead sums in big-bead order, then over big beads (src/md.cpp:606-614) */
    const double shc = s->bb_shc;
    s->bb_ne_tot = s->bb_ce_tot = 0;
    for (int i = 0; i < s->nbb; i++) {
      double bce = 0, bne = 0;
      for (int j = 0; j < n; j++) {
        const double qj = s->b_q[j % np];
        const int electrostatic = (qj != 0);
        double cej = 0.0, nej = 0.0;
        const real r = vnorm(pbc(vsub(s->bb_pos[i], s->pos[j]), bx, hbx));
        const double sig1 = s->bb_sigma, sig2 = s->b_sigma[j % np];
        const double sigavg = (sig1 + sig2) / 2;
        const double delta = sigavg - shc;
        const double shc6 = pow(shc, 6);
        const double r6 = (double)POW(r - delta, (real)6);
        const double yukawa_scale = exp(kappa * sigavg) / ((1 + kappa * sig1 / 2) * (1 + kappa * sig2 / 2));
        if (electrostatic && r < ecut_el) cej = (double)((s->bb_q * qj * lb * EXP(-kappa * r) * yukawa_scale) / (r));
        bce += cej;
        s->ce[j] += cej;
        if (r < delta + 1.12246205 * shc) nej = ((4 * (shc6 / r6) * ((shc6 / r6) - 1)) + 1);
        bne += nej;
        s->ne[j] += nej;
      }
      s->bb_ce_tot += bce;
      s->bb_ne_tot += bne;
    }
  }
  for (int g = 0; g < n; g++) {
    if (se) se[g] = s->se[g];
    if (ke) ke[g] = s->ke[g];
    if (be) be[g] = s->be[g];
    if (neo) neo[g] = s->ne[g];
    if (ce) ce[g] = s->ce[g];
  }
}

/* Thermostat chain set-up, src/md.cpp:187-196 and src/thermostat.h:20-28. */
void oracle_nhc_init(oracle_nhc* c, int chain_len, double q_mass, double temperature, int n_beads) {
  memset(c, 0, sizeof(*c));
  const double T = temperature / (double)298;
  if (chain_len == 1) {
    c->m = 1;
    c->q[0] = 0;
    c->t[0] = T;
    c->dof[0] = 3ul * n_beads;
    return;
  }
  int m = 0;
  c->q[m] = q_mass;
  c->t[m] = T;
  c->dof[m] = 3ul * n_beads;
  m++;
  while (m != chain_len - 1 && m < 15) {
    c->q[m] = 1;
    c->t[m] = T;
    c->dof[m] = 1;
    m++;
  }
  c->q[m] = 0;
  c->t[m] = T;
  c->dof[m] = 3ul * n_beads;
  m++;
  c->m = m;
}

/* update_chain_xi (src/functions.cpp:33-58); ke is a long double parameter. */
static void chain_xi(oracle_nhc* c, int j, double dt, real ke) {
  if (c->q[j] == 0) return;
  const double kB = 1;
  if (j != 0) {
    c->xi[j] = c->xi[j] * exp(-0.5 * dt * c->xi[j + 1]) +
               0.5 * dt * (1.0 / c->q[j]) *
                   (c->q[j - 1] * c->xi[j - 1] * c->xi[j - 1] - c->dof[j] * kB * c->t[j]) *
                   exp(-0.25 * dt * c->xi[j + 1]);
  } else {
    c->xi[j] = (double)(c->xi[j] * exp(-0.5 * dt * c->xi[j + 1]) +
                        0.5 * dt * (1.0 / c->q[j]) * (2 * ke - c->dof[j] * kB * c->t[j]) *
                            exp(-0.25 * dt * c->xi[j + 1]));
  }
}

/* THERMOSTAT::update_eta (src/thermostat.h:35-40) */
static void chain_eta(oracle_nhc* c, int j, double dt) {
  if (c->q[j] == 0) return;
  c->eta[j] = c->eta[j] + 0.5 * dt * c->xi[j];
}

unsigned oracle_loop_end(double steps, double dt) {
  const double totaltime = steps * dt; /* src/md.cpp:137 */
  unsigned a = 0;
  while (a < ((totaltime / dt) + 1)) a++; /* src/md.cpp:387 */
  return a;
}

/* One iteration of the MD loop, molecular-dynamics branch: src/md.cpp:400-514. */
int oracle_md_step(oracle_sys* s, oracle_nhc* c, unsigned a, double dt, int build_freq,
                   double* ke_io, double* vcom_mag) {
  const int n = s->n, np = s->d.np;
  double particle_ke = *ke_io;
  for (int j = c->m - 1; j > -1; j--) chain_xi(c, j, dt, (real)particle_ke);
  for (int j = 0; j < c->m; j++) chain_eta(c, j, dt);
  const double expfac = exp(-0.5 * dt * c->xi[0]);
  for (int g = 0; g < n; g++) {
    const double m = s->b_mass[g % np];
    /* BEAD::therm_update_velocity (src/bead.h:113-117) */
    s->vel[g] = vadd(vscale(s->vel[g], (real)expfac),
                     vscale(s->tforce[g], (real)(0.5 * dt * (sqrt(expfac)) / m)));
    /* BEAD::update_position (src/bead.h:72-81) */
    vec3 p = vadd(s->pos[g], vscale(s->vel[g], (real)dt));
    if (p.x > s->hbx) p.x = p.x - s->bx;
    else if (p.x < -s->hbx) p.x = p.x + s->bx;
    if (p.y > s->hbx) p.y = p.y - s->bx;
    else if (p.y < -s->hbx) p.y = p.y + s->bx;
    if (p.z > s->hbx) p.z = p.z - s->bx;
    else if (p.z < -s->hbx) p.z = p.z + s->bx;
    s->pos[g] = p;
  }
  const int rebuild = (a % (unsigned)build_freq == 0);
  int over = oracle_forces(s, rebuild);
  for (int g = 0; g < n; g++) {
    const double m = s->b_mass[g % np];
    s->vel[g] = vadd(vscale(s->vel[g], (real)expfac),
                     vscale(s->tforce[g], (real)(0.5 * dt * (sqrt(expfac)) / m)));
  }
  particle_ke = (double)kinetic_energy_real(s);
  for (int j = 0; j < c->m; j++) chain_eta(c, j, dt);
  for (int j = 0; j < c->m; j++) chain_xi(c, j, dt, (real)particle_ke);
  vec3 avg = v3(0, 0, 0);
  for (int g = 0; g < n; g++) avg = vadd(avg, s->vel[g]);
  avg = vscale(avg, (real)(1.0 / n));
  for (int g = 0; g < n; g++) s->vel[g] = vsub(s->vel[g], avg);
  *ke_io = particle_ke;
  if (vcom_mag) *vcom_mag = (double)vnorm(avg);
  return over;
}
