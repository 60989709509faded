/* Oracle test infrastructure (the checker and the CPU-baseline timing, never the product).
 *
 * C restatement of the per-frame work of the reference's analyze_output, with the reference's
 * own loop structure so that its cost is the reference's cost:
 *   pair correlation   every bead pair i < j, both of the pcf type, distance < half box, bin
 *                      floor(distance / delta_g)                        (src/analysis.cpp:117-131)
 *   oligomers          grown one at a time from the first unassigned subunit: every subunit
 *                      added last round is tested against every later unassigned subunit,
 *                      bead against bead, and the first pair closer than the contact distance
 *                      adds it                                           (src/analysis.cpp:140-178)
 *   sub-oligomers      inside each oligomer, grown from each unassigned so-type bead over the
 *                      oligomer's so-type beads                          (src/analysis.cpp:189-238)
 *   histograms         oligomers by size, sub-oligomers by (size - 1) / 3 (src/analysis.cpp:180-186,240-245)
 * Distances follow dist() (src/functions.h:42-56) in REAL (long double by default, as the
 * reference's VECTOR3D), with the reference's image rule (half box never set: every nonzero
 * difference shifted by a full box) or the minimum image.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORACLE_REAL
#define ORACLE_REAL long double
#endif
typedef ORACLE_REAL real;

static inline __attribute__((always_inline)) real shift(real x, real L, real h) {
  if (x > h) return x - L;
  if (x < -h) return x + L;
  return x;
}

/* dist(A, B).GetMagnitude() with the half box h: 0 for the reference's analysis (its beads never
 * get a half-box vector), L / 2 for the minimum image. */
static inline __attribute__((always_inline)) real sep(const real* p, long a, long b, real L, real h) {
  const real x = shift(p[3 * a] - p[3 * b], L, h);
  const real y = shift(p[3 * a + 1] - p[3 * b + 1], L, h);
  const real z = shift(p[3 * a + 2] - p[3 * b + 2], L, h);
  return sqrtl(x * x + y * y + z * z);
}

/* One frame.  pos [n][3], types [n]; outputs gr [bins], ms [S], so [2S] (zeroed here).
 * Returns 0, or 1 when a sub-oligomer would land past the so histogram. */
int oracle_analysis_frame(long n, int np, const int* types, const double* pos, double box, int image,
                          int pcf_type, int bins, int so_type, double contact, long long* gr, long long* ms,
                          long long* so) {
  const long S = n / np;
  real* p = (real*)malloc(sizeof(real) * 3 * n);
  for (long i = 0; i < 3 * n; i++) p[i] = pos[i];
  const real L = (real)box;
  const real h = image == 0 ? (real)0 : L / 2;
  const double half = box / 2, delta_g = box / (2.0 * bins);
  memset(gr, 0, sizeof(long long) * bins);
  memset(ms, 0, sizeof(long long) * S);
  memset(so, 0, sizeof(long long) * 2 * S);
  int rc = 0;

  for (long i = 0; i < n; i++)
    for (long j = i + 1; j < n; j++)
      if (types[i] == pcf_type && types[j] == pcf_type) {
        const double distance = (double)sep(p, i, j, L, h);
        if (distance < half) {
          const long k = (long)floor(distance / delta_g);
          if (k < bins) gr[k] += 1;
        }
      }

  /* oligomers: member lists in growth order */
  int* olig_of = (int*)malloc(sizeof(int) * S);
  long* members = (long*)malloc(sizeof(long) * S);
  long* olig_start = (long*)malloc(sizeof(long) * (S + 1));
  long n_olig = 0, n_members = 0;
  for (long s = 0; s < S; s++) olig_of[s] = -1;
  for (long i = 0; i < S; i++) {
    if (olig_of[i] >= 0) continue;
    const long start = n_members;
    olig_start[n_olig] = start;
    members[n_members++] = i;
    olig_of[i] = (int)n_olig;
    long oldsize = 0;
    while (oldsize < n_members - start) {
      const long grown_from = oldsize;
      oldsize = n_members - start;
      for (long j = grown_from; j < oldsize; j++) {
        const long g = members[start + j];
        for (long k = i + 1; k < S; k++) {
          if (olig_of[k] >= 0) continue;
          int hit = 0;
          for (int m = 0; m < np && !hit; m++)
            for (int q = 0; q < np; q++)
              if (sep(p, g * np + m, k * np + q, L, h) < contact) {
                hit = 1;
                break;
              }
          if (hit) {
            members[n_members++] = k;
            olig_of[k] = (int)n_olig;
          }
        }
      }
    }
    n_olig++;
  }
  olig_start[n_olig] = n_members;
  for (long o = 0; o < n_olig; o++) ms[olig_start[o + 1] - olig_start[o] - 1] += 1;

  /* sub-oligomers inside each oligomer */
  char* in_so = (char*)calloc(n, 1);
  long* sob = (long*)malloc(sizeof(long) * n);
  for (long o = 0; o < n_olig; o++) {
    for (long j = olig_start[o]; j < olig_start[o + 1]; j++) {
      for (int jj = 0; jj < np; jj++) {
        const long b0 = members[j] * np + jj;
        if (in_so[b0] || types[b0] != so_type) continue;
        long cnt = 0;
        sob[cnt++] = b0;
        in_so[b0] = 1;
        long oldsize = 0;
        while (oldsize < cnt) {
          const long grown_from = oldsize;
          oldsize = cnt;
          for (long gidx = grown_from; gidx < oldsize; gidx++) {
            const long g = sob[gidx];
            for (long k = olig_start[o]; k < olig_start[o + 1]; k++)
              for (int kk = 0; kk < np; kk++) {
                const long b = members[k] * np + kk;
                if (in_so[b] || types[b] != so_type) continue;
                if (sep(p, g, b, L, h) < contact) {
                  sob[cnt++] = b;
                  in_so[b] = 1;
                }
              }
          }
        }
        const long bin = (cnt - 1) / 3;
        if (bin < 2 * S) so[bin] += 1;
        else rc = 1;
      }
    }
  }
  free(in_so);
  free(sob);
  free(olig_of);
  free(members);
  free(olig_start);
  free(p);
  return rc;
}
