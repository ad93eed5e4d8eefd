/*
 * CPU oracle for the stochastic LLG step (TEST INFRASTRUCTURE ONLY; see
 * llg_oracle.h for the list of reference routines restated here).
 *
 * Build: gcc -std=c11 -O2 -fopenmp -ffp-contract=off -fPIC -shared
 *
 * Everything is FP64 and evaluated in the association order of the reference
 * source; the comments above each routine give the file:line it follows.
 */
#define _POSIX_C_SOURCE 200809L
#include "llg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* src/jams/helpers/consts.h:32 */
static const double kBoltzmannIU = 0.0861733326;
/* src/jams/helpers/consts.h:35,38: mu0 in internal units (4 pi 1e-7 / kJoule2meV) */
static const double kPi = 3.14159265358979323846;
static const double kJoule2meV = 6.24150907e21;

static char g_err[512];

static int fail(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return -1;
}

const char *orc_last_error(void) { return g_err; }

void orc_set_threads(int32_t n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Gaussian noise: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel      */
/* random numbers: as easy as 1, 2, 3", SC'11) + Box-Muller.  The log and    */
/* sin/cos are series written out here with single-precision fused          */
/* multiply-adds, so the GPU library can produce the identical floats.      */
/* ------------------------------------------------------------------------ */

static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0;
    uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

static float bits_to_float(uint32_t b) {
  float f;
  memcpy(&f, &b, 4);
  return f;
}
static uint32_t float_to_bits(float f) {
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
}

/* natural log of u in (0, 1]: u = m 2^e with m in (sqrt(1/2), sqrt(2)],
   ln m = 2 atanh(f), f = (m - 1)/(m + 1), atanh series to f^9 */
static float noise_log(float u) {
  uint32_t b = float_to_bits(u);
  int32_t e = (int32_t)(b >> 23) - 127;
  uint32_t mb = (b & 0x007FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) { /* m > sqrt(2) */
    mb -= 0x00800000u;    /* m / 2 */
    e += 1;
  }
  float m = bits_to_float(mb);
  float f = (m - 1.0f) / (m + 1.0f);
  float f2 = f * f;
  float p = 0x1.c71c72p-4f;                 /* 1/9 */
  p = fmaf(p, f2, 0x1.24924ap-3f);          /* 1/7 */
  p = fmaf(p, f2, 0x1.99999ap-3f);          /* 1/5 */
  p = fmaf(p, f2, 0x1.555556p-2f);          /* 1/3 */
  p = fmaf(p, f2, 1.0f);
  float lnm = 2.0f * (f * p);
  return fmaf((float)e, 0x1.62e430p-1f, lnm); /* e ln 2 + ln m */
}

/* sin and cos of 2 pi k / 2^24 for a 24-bit integer k */
static void noise_sincos(uint32_t k, float *s_out, float *c_out) {
  uint32_t q = k >> 22;
  int32_t j = (int32_t)(k & 0x3FFFFFu);
  if (j >= (1 << 21)) {
    q += 1;
    j -= (1 << 22);
  }
  float r = (float)j * 0x1.0p-22f;  /* in [-1/2, 1/2): angle = pi/2 (q + r) */
  float r2 = r * r;
  float sp = 0x1.507834p-13f;
  sp = fmaf(sp, r2, -0x1.32d2ccp-8f);
  sp = fmaf(sp, r2, 0x1.466bc6p-4f);
  sp = fmaf(sp, r2, -0x1.4abbcep-1f);
  sp = fmaf(sp, r2, 0x1.921fb6p+0f);
  float sn = sp * r;
  float cp = 0x1.e1f506p-11f;
  cp = fmaf(cp, r2, -0x1.55d3c8p-6f);
  cp = fmaf(cp, r2, 0x1.03c1f0p-2f);
  cp = fmaf(cp, r2, -0x1.3bd3ccp+0f);
  float cs = fmaf(cp, r2, 1.0f);
  switch (q & 3u) {
    case 0: *s_out = sn; *c_out = cs; break;
    case 1: *s_out = cs; *c_out = -sn; break;
    case 2: *s_out = -sn; *c_out = -cs; break;
    default: *s_out = -cs; *c_out = sn; break;
  }
}

void orc_noise_normals(uint64_t seed, uint32_t replica, uint64_t step,
                       uint32_t spin, float out[3]) {
  uint32_t c[4] = {spin, replica, (uint32_t)step, (uint32_t)(step >> 32)};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  float u1 = (float)((c[0] >> 8) + 1u) * 0x1.0p-24f; /* (0, 1] */
  float u2 = (float)((c[2] >> 8) + 1u) * 0x1.0p-24f;
  float r1 = sqrtf(-2.0f * noise_log(u1));
  float r2 = sqrtf(-2.0f * noise_log(u2));
  float s1, c1, s2, c2;
  noise_sincos(c[1] >> 8, &s1, &c1);
  noise_sincos(c[3] >> 8, &s2, &c2);
  out[0] = r1 * c1;
  out[1] = r1 * s1;
  out[2] = r2 * c2;
  (void)s2;
}

/* ------------------------------------------------------------------------ */
/* model                                                                     */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t *rows; /* 3N + 1 */
  int32_t *cols;
  double *vals;
  int64_t nnz;
} csr_t;

/* dipole term: for basis site b, entries start[b] .. start[b+1]-1 of the
   source sites (basis bj at cell offset d) within the cutoff and their
   tensors w (xx, xy, xz, yy, yz, zz) x mu0 / (4 pi a^3) */
typedef struct {
  int32_t bj;
  int32_t d[3];
  double w[6];
} dip_entry_t;

typedef struct {
  int64_t start[9];   /* nb + 1 <= 9 */
  dip_entry_t *e;
} dip_t;

struct orc_sim {
  orc_model m;
  int64_t n;
  int32_t nt;
  orc_term *terms;
  csr_t *csr;        /* one per term (only exchange terms are filled) */
  dip_t *dip;        /* one per term (only dipole terms are filled) */
  /* per-spin parameter arrays, as globals::mus/gyro/alpha */
  double *mus, *gyro, *alpha, *sigma;
  /* scratch */
  double *h, *h2, *w, *s_old, *ds, *k1, *k2, *k3, *k4, *tmp;
};

int64_t orc_num_spins(const orc_sim *s) { return s->n; }

static inline int64_t site_index(const orc_sim *s, int64_t i, int64_t j,
                                 int64_t k, int64_t b) {
  return ((i * s->m.L[1] + j) * s->m.L[2] + k) * s->m.nb + b;
}

typedef struct {
  int32_t j;
  int32_t e;
} nbr_t;

static int cmp_nbr(const void *a, const void *b) {
  const nbr_t *x = (const nbr_t *)a, *y = (const nbr_t *)b;
  if (x->j != y->j) return x->j < y->j ? -1 : 1;
  return 0;
}

/* Neighbour list + CSR for one exchange term.
   Loop order and boundary rule: src/jams/core/interactions.cc:350-396 and
   src/jams/core/lattice.cc:987-1007; a site pair reached twice is an error
   (interactions.cc:371-380).  Entries: insert_interaction_tensor
   (sparse_interaction.cc:25-34) for tensors with max|J| > 0 (exchange.cc:
   162-169), then sorted by (row, col) (sparse_matrix_builder.h:108-145). */
static int build_exchange_csr(orc_sim *s, const orc_term *t, csr_t *out) {
  const int64_t n = s->n;
  const int32_t nb = s->m.nb;
  int32_t *per_b = calloc((size_t)nb, sizeof(int32_t));
  for (int e = 0; e < t->n_int; ++e) {
    if (t->bi[e] < 0 || t->bi[e] >= nb || t->bj[e] < 0 || t->bj[e] >= nb) {
      free(per_b);
      return fail("exchange entry %d has a basis index outside [0, %d)", e, nb);
    }
    per_b[t->bi[e]]++;
  }
  int32_t zmax = 0;
  for (int b = 0; b < nb; ++b) zmax = per_b[b] > zmax ? per_b[b] : zmax;
  free(per_b);

  out->rows = calloc((size_t)(3 * n + 1), sizeof(int64_t));
  /* count pass: nonzeros per row */
  int64_t *row_count = calloc((size_t)(3 * n), sizeof(int64_t));
  int err = 0;
  nbr_t *list = malloc(sizeof(nbr_t) * (size_t)(zmax > 0 ? zmax : 1));
  int pass;
  for (pass = 0; pass < 2 && !err; ++pass) {
    if (pass == 1) {
      out->rows[0] = 0;
      for (int64_t r = 0; r < 3 * n; ++r) out->rows[r + 1] = out->rows[r] + row_count[r];
      out->nnz = out->rows[3 * n];
      out->cols = malloc(sizeof(int32_t) * (size_t)(out->nnz > 0 ? out->nnz : 1));
      out->vals = malloc(sizeof(double) * (size_t)(out->nnz > 0 ? out->nnz : 1));
      memset(row_count, 0, sizeof(int64_t) * (size_t)(3 * n));
    }
    for (int64_t ci = 0; ci < s->m.L[0] && !err; ++ci)
      for (int64_t cj = 0; cj < s->m.L[1] && !err; ++cj)
        for (int64_t ck = 0; ck < s->m.L[2] && !err; ++ck)
          for (int32_t b = 0; b < nb && !err; ++b) {
            int64_t i = site_index(s, ci, cj, ck, b);
            int cnt = 0;
            for (int e = 0; e < t->n_int; ++e) {
              if (t->bi[e] != b) continue;
              int64_t d[3] = {ci + t->T[3 * e], cj + t->T[3 * e + 1], ck + t->T[3 * e + 2]};
              int outside = 0;
              for (int l = 0; l < 3; ++l) {
                if (!s->m.periodic[l] && (d[l] < 0 || d[l] >= s->m.L[l])) {
                  outside = 1;
                  break;
                }
                if (d[l] + s->m.L[l] < 0) {
                  err = fail("interaction translation %lld along axis %d exceeds the lattice size",
                             (long long)t->T[3 * e + l], l);
                  break;
                }
                d[l] = (d[l] + s->m.L[l]) % s->m.L[l];
              }
              if (err) break;
              if (outside) continue;
              list[cnt].j = (int32_t)site_index(s, d[0], d[1], d[2], t->bj[e]);
              list[cnt].e = e;
              cnt++;
            }
            if (err) break;
            qsort(list, (size_t)cnt, sizeof(nbr_t), cmp_nbr);
            for (int q = 1; q < cnt; ++q) {
              if (list[q].j == list[q - 1].j) {
                err = fail("Multiple interactions for sites %lld and %d", (long long)i, list[q].j);
                break;
              }
            }
            if (err) break;
            for (int q = 0; q < cnt; ++q) {
              const double *J = t->J + 9 * list[q].e;
              double mx = 0.0;
              for (int a = 0; a < 9; ++a) mx = fabs(J[a]) > mx ? fabs(J[a]) : mx;
              if (!(mx > 0.0)) continue;
              for (int mm = 0; mm < 3; ++mm)
                for (int nn = 0; nn < 3; ++nn) {
                  if (J[3 * mm + nn] == 0.0) continue;
                  int64_t r = 3 * i + mm;
                  if (pass == 0) {
                    row_count[r]++;
                  } else {
                    int64_t at = out->rows[r] + row_count[r]++;
                    out->cols[at] = 3 * list[q].j + nn;
                    out->vals[at] = J[3 * mm + nn];
                  }
                }
            }
          }
  }
  free(list);
  free(row_count);
  return err;
}

/* inradius of the periodic part of the supercell (lattice parameters):
   jams::maximum_interaction_length, src/jams/core/lattice.cc:1155-1200 */
static double cross_norm(const double *a, const double *b) {
  const double c0 = a[1] * b[2] - a[2] * b[1], c1 = a[2] * b[0] - a[0] * b[2], c2 = a[0] * b[1] - a[1] * b[0];
  return sqrt(c0 * c0 + c1 * c1 + c2 * c2);
}

static double vnorm(const double *a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

static double max_interaction_radius(const orc_model *m, const double *A) {
  double v[3][3];
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) v[k][c] = m->L[k] * A[3 * k + c];
  const int p0 = m->periodic[0] != 0, p1 = m->periodic[1] != 0, p2 = m->periodic[2] != 0;
  if (p0 && p1 && p2) {
    const double c0 = v[1][1] * v[2][2] - v[1][2] * v[2][1], c1 = v[1][2] * v[2][0] - v[1][0] * v[2][2],
                 c2 = v[1][0] * v[2][1] - v[1][1] * v[2][0];
    const double vol = fabs(v[0][0] * c0 + v[0][1] * c1 + v[0][2] * c2);
    double h = vol / cross_norm(v[1], v[2]);
    if (vol / cross_norm(v[2], v[0]) < h) h = vol / cross_norm(v[2], v[0]);
    if (vol / cross_norm(v[0], v[1]) < h) h = vol / cross_norm(v[0], v[1]);
    return 0.5 * h;
  }
  if (p0 + p1 + p2 == 2) {
    const double *a = p0 ? v[0] : v[1];
    const double *b = p2 ? v[2] : v[1];
    const double area = cross_norm(a, b);
    const double h1 = area / vnorm(a), h2 = area / vnorm(b);
    return 0.5 * (h1 < h2 ? h1 : h2);
  }
  if (p0 + p1 + p2 == 1) return 0.5 * vnorm(p0 ? v[0] : (p1 ? v[1] : v[2]));
  double d[3] = {v[0][0] + v[1][0] + v[2][0], v[0][1] + v[1][1] + v[2][1], v[0][2] + v[1][2] + v[2][2]};
  return vnorm(d);
}

/* every source site within r_cutoff + distance_tolerance of each basis site:
   the real-space tensor the reference's FFT term builds
   (src/jams/hamiltonian/dipole_fft.cc:205-265), listed per target site */
static int build_dipole(orc_sim *s, const orc_term *tm, dip_t *out) {
  const orc_model *m = &s->m;
  if (m->nb > 8) return fail("dipole: at most 8 basis sites");
  if (!tm->lattice_vectors || !tm->positions || !(tm->lattice_parameter > 0.0) || !(tm->r_cutoff > 0.0))
    return fail("dipole: lattice vectors, positions, lattice parameter and r_cutoff are required");
  const double *A = tm->lattice_vectors;
  if (tm->r_cutoff > max_interaction_radius(m, A))
    return fail("dipole: r_cutoff is larger than the inradius of the periodic supercell");
  const double rc = tm->r_cutoff + tm->distance_tolerance;
  const double a = tm->lattice_parameter;
  const double w0 = (4.0 * kPi * 1e-7 / kJoule2meV) / (4.0 * kPi * a * a * a);
  int lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = m->periodic[k] ? 0 : -(m->L[k] - 1);
    hi[k] = m->L[k] - 1;
  }
  size_t cap = 1024, n = 0;
  out->e = malloc(cap * sizeof(dip_entry_t));
  for (int bi = 0; bi < m->nb; ++bi) {
    out->start[bi] = (int64_t)n;
    const double *fi = tm->positions + 3 * bi;
    for (int bj = 0; bj < m->nb; ++bj) {
      const double *fj = tm->positions + 3 * bj;
      for (int d0 = lo[0]; d0 <= hi[0]; ++d0)
        for (int d1 = lo[1]; d1 <= hi[1]; ++d1)
          for (int d2 = lo[2]; d2 <= hi[2]; ++d2) {
            const int d[3] = {d0, d1, d2};
            if (d0 == 0 && d1 == 0 && d2 == 0 && bi == bj) continue;   /* self */
            double x[3];
            for (int k = 0; k < 3; ++k) {
              x[k] = d[k] + fj[k] - fi[k];
              if (m->periodic[k]) x[k] -= m->L[k] * floor(x[k] / m->L[k] + 0.5);
            }
            double r[3];
            for (int c = 0; c < 3; ++c) r[c] = x[0] * A[c] + x[1] * A[3 + c] + x[2] * A[6 + c];
            const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            if (!(r2 > 0.0)) return fail("dipole: two sites at the same position");
            if (r2 > rc * rc) continue;
            const double r5 = pow(sqrt(r2), 5);
            if (n == cap) {
              cap *= 2;
              out->e = realloc(out->e, cap * sizeof(dip_entry_t));
            }
            dip_entry_t *e = &out->e[n++];
            e->bj = bj;
            for (int k = 0; k < 3; ++k) e->d[k] = d[k];
            e->w[0] = w0 * (3.0 * r[0] * r[0] - r2) / r5;
            e->w[1] = w0 * (3.0 * r[0] * r[1]) / r5;
            e->w[2] = w0 * (3.0 * r[0] * r[2]) / r5;
            e->w[3] = w0 * (3.0 * r[1] * r[1] - r2) / r5;
            e->w[4] = w0 * (3.0 * r[1] * r[2]) / r5;
            e->w[5] = w0 * (3.0 * r[2] * r[2] - r2) / r5;
          }
    }
  }
  out->start[m->nb] = (int64_t)n;
  return 0;
}

void orc_destroy(orc_sim *s) {
  if (!s) return;
  if (s->csr) {
    for (int t = 0; t < s->nt; ++t) {
      free(s->csr[t].rows);
      free(s->csr[t].cols);
      free(s->csr[t].vals);
    }
    free(s->csr);
  }
  if (s->dip) {
    for (int t = 0; t < s->nt; ++t) free(s->dip[t].e);
    free(s->dip);
  }
  free(s->terms);
  free(s->mus); free(s->gyro); free(s->alpha); free(s->sigma);
  free(s->h); free(s->h2); free(s->w); free(s->s_old); free(s->ds);
  free(s->k1); free(s->k2); free(s->k3); free(s->k4); free(s->tmp);
  free(s);
}

int orc_create(const orc_model *m, orc_sim **out) {
  *out = NULL;
  if (m->nb < 1) return fail("need at least one basis site");
  for (int l = 0; l < 3; ++l)
    if (m->L[l] < 1) return fail("lattice size must be positive");
  if (m->n_terms < 0 || (m->n_terms > 0 && !m->terms)) return fail("bad term list");
  orc_sim *s = calloc(1, sizeof(orc_sim));
  s->m = *m;
  s->n = (int64_t)m->L[0] * m->L[1] * m->L[2] * m->nb;
  if (3 * s->n >= (int64_t)INT32_MAX) {
    free(s);
    return fail("lattice too large for the oracle");
  }
  s->nt = m->n_terms;
  s->terms = calloc((size_t)(s->nt > 0 ? s->nt : 1), sizeof(orc_term));
  memcpy(s->terms, m->terms, sizeof(orc_term) * (size_t)s->nt);
  s->csr = calloc((size_t)(s->nt > 0 ? s->nt : 1), sizeof(csr_t));
  s->dip = calloc((size_t)(s->nt > 0 ? s->nt : 1), sizeof(dip_t));
  const int64_t n = s->n, n3 = 3 * n;
  s->mus = malloc(sizeof(double) * n);
  s->gyro = malloc(sizeof(double) * n);
  s->alpha = malloc(sizeof(double) * n);
  s->sigma = malloc(sizeof(double) * n);
  for (int64_t i = 0; i < n; ++i) {
    int b = (int)(i % m->nb);
    s->mus[i] = m->mus[b];
    s->gyro[i] = m->gyro[b];
    s->alpha[i] = m->alpha[b];
    /* src/jams/solvers/cpu_llg_heun.cc:36-43 */
    double denominator = 1.0;
    if (m->gilbert_prefactor) denominator = 1.0 + s->alpha[i] * s->alpha[i];
    s->sigma[i] = sqrt((2.0 * kBoltzmannIU * s->alpha[i]) /
                       (s->mus[i] * s->gyro[i] * m->dt * denominator));
  }
  for (int t = 0; t < s->nt; ++t) {
    const orc_term *tm = &s->terms[t];
    if (tm->kind == ORC_TERM_EXCHANGE) {
      if (build_exchange_csr(s, tm, &s->csr[t]) != 0) {
        orc_destroy(s);
        return -1;
      }
    } else if (tm->kind == ORC_TERM_UNIAXIAL) {
      if (!(tm->order == 2 || tm->order == 4 || tm->order == 6)) {
        orc_destroy(s);
        return fail("uniaxial power must be 2, 4 or 6");
      }
    } else if (tm->kind == ORC_TERM_CUBIC) {
      if (!(tm->order == 1 || tm->order == 2)) {
        orc_destroy(s);
        return fail("cubic order must be 1 or 2");
      }
    } else if (tm->kind == ORC_TERM_DIPOLE) {
      if (build_dipole(s, tm, &s->dip[t]) != 0) {
        orc_destroy(s);
        return -1;
      }
    } else if (tm->kind == ORC_TERM_ZEEMAN) {
      if (!tm->dc_field || (tm->ac_field && !tm->ac_frequency)) {
        orc_destroy(s);
        return fail("zeeman: dc field per basis site, ac field with its frequency");
      }
    } else if (tm->kind == ORC_TERM_APPLIED_FIELD) {
      if (tm->pulse < ORC_PULSE_STATIC || tm->pulse > ORC_PULSE_SINC_COS) {
        orc_destroy(s);
        return fail("unknown field pulse type %d", tm->pulse);
      }
    } else {
      orc_destroy(s);
      return fail("unknown term kind %d", tm->kind);
    }
  }
  s->h = malloc(sizeof(double) * n3);
  s->h2 = malloc(sizeof(double) * n3);
  s->w = calloc((size_t)n3, sizeof(double));
  s->s_old = malloc(sizeof(double) * n3);
  s->ds = malloc(sizeof(double) * n3);
  s->k1 = malloc(sizeof(double) * n3);
  s->k2 = malloc(sizeof(double) * n3);
  s->k3 = malloc(sizeof(double) * n3);
  s->k4 = malloc(sizeof(double) * n3);
  s->tmp = malloc(sizeof(double) * n3);
  *out = s;
  return 0;
}

int orc_exchange_csr(const orc_sim *s, int32_t term, int64_t *nnz,
                     const int64_t **rows, const int32_t **cols,
                     const double **vals) {
  if (term < 0 || term >= s->nt || s->terms[term].kind != ORC_TERM_EXCHANGE)
    return fail("term %d is not an exchange term", term);
  *nnz = s->csr[term].nnz;
  *rows = s->csr[term].rows;
  *cols = s->csr[term].cols;
  *vals = s->csr[term].vals;
  return 0;
}

double orc_sigma(const orc_sim *s, int32_t b) { return s->sigma[b]; }

/* ------------------------------------------------------------------------ */
/* fields                                                                    */
/* ------------------------------------------------------------------------ */

/* sinc(x) = sin(x) / x, 1 at 0 (src/jams/helpers/maths.h:437-446) */
static double sinc_ref(double x) {
  if (x == 0.0) return 1.0;
  return sin(x) / x;
}

/* one term's field at spin i and solver time `time` (ps) into f[3] */
static void term_field(const orc_sim *s, int t, const double *spins, int64_t i,
                       double time, double f[3]) {
  const orc_term *tm = &s->terms[t];
  const int b = (int)(i % s->m.nb);
  const double *sp = spins + 3 * i;
  switch (tm->kind) {
    case ORC_TERM_EXCHANGE: {
      /* Xcsrmv_general_row: src/jams/interface/sparse_blas.h:13-27 */
      const csr_t *c = &s->csr[t];
      for (int mm = 0; mm < 3; ++mm) {
        int64_t r = 3 * i + mm;
        double sum = 0.0;
        for (int64_t e = c->rows[r]; e < c->rows[r + 1]; ++e) sum += spins[c->cols[e]] * c->vals[e];
        f[mm] = sum;
      }
      break;
    }
    case ORC_TERM_UNIAXIAL: {
      /* src/jams/hamiltonian/uniaxial_anisotropy.cc:155-163 */
      const double *a = tm->axis + 3 * b;
      double dot = (a[0] * sp[0] + a[1] * sp[1] + a[2] * sp[2]);
      for (int j = 0; j < 3; ++j)
        f[j] = tm->K[b] * tm->order * pow(dot, tm->order - 1) * a[j];
      break;
    }
    case ORC_TERM_CUBIC: {
      /* src/jams/hamiltonian/cubic_anisotropy.cc:197-226 */
      const double *u = tm->axis + 9 * b, *v = u + 3, *w = u + 6;
      double Su = sp[0] * u[0] + sp[1] * u[1] + sp[2] * u[2];
      double Sv = sp[0] * v[0] + sp[1] * v[1] + sp[2] * v[2];
      double Sw = sp[0] * w[0] + sp[1] * w[1] + sp[2] * w[2];
      double pre = 2.0 * tm->K[b];
      for (int j = 0; j < 3; ++j) {
        double fj = 0.0;
        if (tm->order == 1) {
          fj += pre * (u[j] * Su * (Sv * Sv + Sw * Sw) + v[j] * Sv * (Sw * Sw + Su * Su) +
                       w[j] * Sw * (Su * Su + Sv * Sv));
        } else {
          fj += pre * (u[j] * Su * (Sv * Sv) * (Sw * Sw) + v[j] * Sv * (Sw * Sw) * (Su * Su) +
                       w[j] * Sw * (Su * Su) * (Sv * Sv));
        }
        f[j] = fj;
      }
      break;
    }
    case ORC_TERM_DIPOLE: {
      /* h_i = mu_i sum_j mu_j w_ij . s_j (dipole_bruteforce.cc:96-116) */
      const dip_t *dp = &s->dip[t];
      const int64_t ci = i / s->m.nb;
      int c[3];
      c[2] = (int)(ci % s->m.L[2]);
      c[1] = (int)((ci / s->m.L[2]) % s->m.L[1]);
      c[0] = (int)(ci / ((int64_t)s->m.L[2] * s->m.L[1]));
      double acc[3] = {0.0, 0.0, 0.0};
      for (int64_t k = dp->start[b]; k < dp->start[b + 1]; ++k) {
        const dip_entry_t *e = &dp->e[k];
        int cj[3], ok = 1;
        for (int l = 0; l < 3; ++l) {
          cj[l] = c[l] + e->d[l];
          if (s->m.periodic[l]) cj[l] = ((cj[l] % s->m.L[l]) + s->m.L[l]) % s->m.L[l];
          else if (cj[l] < 0 || cj[l] >= s->m.L[l]) ok = 0;
        }
        if (!ok) continue;
        const int64_t j = site_index(s, cj[0], cj[1], cj[2], e->bj);
        const double *sj = spins + 3 * j;
        const double muj = s->mus[j];
        acc[0] += muj * (e->w[0] * sj[0] + e->w[1] * sj[1] + e->w[2] * sj[2]);
        acc[1] += muj * (e->w[1] * sj[0] + e->w[3] * sj[1] + e->w[4] * sj[2]);
        acc[2] += muj * (e->w[2] * sj[0] + e->w[4] * sj[1] + e->w[5] * sj[2]);
      }
      for (int l = 0; l < 3; ++l) f[l] = s->mus[i] * acc[l];
      break;
    }
    case ORC_TERM_ZEEMAN: {
      /* dc_local_field = dc mu_s, ac_local_field = ac mu_s, frequency 2 pi f
         (zeeman.cc:26-71); field = dc_local + ac_local cos(w t) (:106-121) */
      for (int j = 0; j < 3; ++j) {
        double fj = tm->dc_field[3 * b + j] * s->mus[i];
        if (tm->ac_field) {
          const double w = 2.0 * kPi * tm->ac_frequency[b];
          fj += (tm->ac_field[3 * b + j] * s->mus[i]) * cos(w * time);
        }
        f[j] = fj;
      }
      break;
    }
    default: { /* ORC_TERM_APPLIED_FIELD: src/jams/hamiltonian/applied_field.cc:10-103,146-148 */
      double B[3] = {tm->B[0], tm->B[1], tm->B[2]};
      if (tm->pulse != ORC_PULSE_STATIC) {
        /* SincField / SincCosField::field: B sinc(pi f_bw (t - t0)) [cos(2 pi f_c (t - t0))] */
        const double sv = sinc_ref(kPi * tm->freq_bandwidth * (time - tm->time_center));
        for (int j = 0; j < 3; ++j) B[j] = B[j] * sv;
        if (tm->pulse == ORC_PULSE_SINC_COS) {
          const double cv = cos(2.0 * kPi * tm->freq_center * (time - tm->time_center));
          for (int j = 0; j < 3; ++j) B[j] = B[j] * cv;
        }
      }
      for (int j = 0; j < 3; ++j) f[j] = s->mus[i] * B[j];
      break;
    }
  }
}

/* Solver::compute_fields: copy of term 0 then daxpy(1.0) of the others
   (src/jams/core/solver.cc:43-57) */
static void compute_fields(const orc_sim *s, const double *spins, double time, double *h) {
  const int64_t n = s->n;
  if (s->nt == 0) {
    memset(h, 0, sizeof(double) * 3 * n);
    return;
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double f[3];
    term_field(s, 0, spins, i, time, f);
    double acc[3] = {f[0], f[1], f[2]};
    for (int t = 1; t < s->nt; ++t) {
      term_field(s, t, spins, i, time, f);
      for (int j = 0; j < 3; ++j) acc[j] += 1.0 * f[j];
    }
    for (int j = 0; j < 3; ++j) h[3 * i + j] = acc[j];
  }
}

int orc_fields(orc_sim *s, const double *spins, double t, double *h) {
  compute_fields(s, spins, t, h);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* integrators                                                               */
/* ------------------------------------------------------------------------ */

static void draw_noise(orc_sim *s, uint64_t step) {
  const int64_t n = s->n;
  const double sqrt_temperature = sqrt(s->m.temperature);
  if (s->m.serial_noise) {
    for (int64_t i = 0; i < n; ++i) {
      float z[3];
      orc_noise_normals(s->m.seed, s->m.replica, step, (uint32_t)i, z);
      for (int j = 0; j < 3; ++j) s->w[3 * i + j] = (double)z[j] * s->sigma[i] * sqrt_temperature;
    }
  } else {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      float z[3];
      orc_noise_normals(s->m.seed, s->m.replica, step, (uint32_t)i, z);
      for (int j = 0; j < 3; ++j) s->w[3 * i + j] = (double)z[j] * s->sigma[i] * sqrt_temperature;
    }
  }
}

/* h <- w + h / mu_s (T > 0) or h / mu_s  (cpu_llg_heun.cc:67-81) */
static void scale_field(orc_sim *s, double *h, int thermal) {
  const int64_t n = s->n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) {
      if (thermal) h[3 * i + j] = (s->w[3 * i + j] + h[3 * i + j] / s->mus[i]);
      else h[3 * i + j] = h[3 * i + j] / s->mus[i];
    }
}

/* rhs = -gamma (S x H + alpha S x (S x H))  (cpu_llg_heun.cc:88) */
static inline void llg_rhs(double g, double a, const double *sp, const double *hh,
                           double rhs[3]) {
  double c1[3] = {sp[1] * hh[2] - sp[2] * hh[1], sp[2] * hh[0] - sp[0] * hh[2],
                  sp[0] * hh[1] - sp[1] * hh[0]};
  double c2[3] = {sp[1] * c1[2] - sp[2] * c1[1], sp[2] * c1[0] - sp[0] * c1[2],
                  sp[0] * c1[1] - sp[1] * c1[0]};
  double mg = -g;
  for (int j = 0; j < 3; ++j) rhs[j] = mg * (c1[j] + a * c2[j]);
}

/* unit_vector: src/jams/containers/vec3.h:275-283 */
static inline void unit_vector(double v[3]) {
  const double length = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (fabs(length) <= DBL_EPSILON) return;
  for (int j = 0; j < 3; ++j) v[j] = v[j] / length;
}

/* HeunLLGSolver::run: src/jams/solvers/cpu_llg_heun.cc:45-148; fields at
   t0 = iteration * dt, then at t0 + dt */
static void heun_step(orc_sim *s, double *spins, uint64_t step) {
  const int64_t n = s->n, n3 = 3 * n;
  const double dt = s->m.dt;
  const double t0 = (double)step * dt;
  const int thermal = s->m.temperature > 0.0;
  memcpy(s->s_old, spins, sizeof(double) * n3);
  if (thermal) draw_noise(s, step);
  compute_fields(s, spins, t0, s->h);
  scale_field(s, s->h, thermal);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double rhs[3];
    llg_rhs(s->gyro[i], s->alpha[i], spins + 3 * i, s->h + 3 * i, rhs);
    double v[3];
    for (int j = 0; j < 3; ++j) {
      s->ds[3 * i + j] = 0.5 * rhs[j];
      v[j] = spins[3 * i + j] + dt * rhs[j];
    }
    unit_vector(v);
    for (int j = 0; j < 3; ++j) spins[3 * i + j] = v[j];
  }
  compute_fields(s, spins, t0 + dt, s->h);
  scale_field(s, s->h, thermal);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double rhs[3];
    llg_rhs(s->gyro[i], s->alpha[i], spins + 3 * i, s->h + 3 * i, rhs);
    double v[3];
    for (int j = 0; j < 3; ++j) {
      s->ds[3 * i + j] = s->ds[3 * i + j] + 0.5 * rhs[j];
      v[j] = s->s_old[3 * i + j] + dt * s->ds[3 * i + j];
    }
    unit_vector(v);
    for (int j = 0; j < 3; ++j) spins[3 * i + j] = v[j];
  }
}

/* k = -gamma (S x H' + alpha S x (S x H')), H' = H / mu_s + noise
   (src/jams/solvers/cuda_llg_rk4_kernel.cuh:26-53) */
static void rk4_derivative(orc_sim *s, const double *spins, double time, double *k, int thermal) {
  const int64_t n = s->n;
  compute_fields(s, spins, time, s->h);
  scale_field(s, s->h, thermal);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) llg_rhs(s->gyro[i], s->alpha[i], spins + 3 * i, s->h + 3 * i, k + 3 * i);
}

/* CudaRK4BaseSolver::run (src/jams/solvers/cuda_rk4_base.cu:50-108) on the
   host: stages s_old + c dt k (cublasDcopy + cublasDaxpy), combination
   s_old + dt (k1 + 2 k2 + 2 k3 + k4) / 6 (cuda_rk4_base_kernel.cuh:14-16),
   then normalise (cuda_spin_ops.cu:4-16, with s / |s| in place of the
   device's approximate reciprocal square root).  Stage times t0, t0 + dt/2,
   t0 + dt/2, t0 + dt (cuda_rk4_base.cu:53-88). */
static void rk4_step(orc_sim *s, double *spins, uint64_t step) {
  const int64_t n = s->n, n3 = 3 * n;
  const double dt = s->m.dt;
  const double t0 = (double)step * dt;
  const int thermal = s->m.temperature > 0.0;
  memcpy(s->s_old, spins, sizeof(double) * n3);
  if (thermal) draw_noise(s, step);
  rk4_derivative(s, spins, t0, s->k1, thermal);
  double c = 0.5 * dt;
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n3; ++q) s->tmp[q] = s->s_old[q] + c * s->k1[q];
  rk4_derivative(s, s->tmp, t0 + 0.5 * dt, s->k2, thermal);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n3; ++q) s->tmp[q] = s->s_old[q] + c * s->k2[q];
  rk4_derivative(s, s->tmp, t0 + 0.5 * dt, s->k3, thermal);
  c = dt;
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n3; ++q) s->tmp[q] = s->s_old[q] + c * s->k3[q];
  rk4_derivative(s, s->tmp, t0 + dt, s->k4, thermal);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double v[3];
    for (int j = 0; j < 3; ++j) {
      int64_t q = 3 * i + j;
      v[j] = s->s_old[q] + dt * (s->k1[q] + 2 * s->k2[q] + 2 * s->k3[q] + s->k4[q]) / 6.0;
    }
    const double len = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int j = 0; j < 3; ++j) spins[3 * i + j] = v[j] / len;
  }
}

int orc_run(orc_sim *s, double *spins, int64_t first_step, int32_t nsteps) {
  for (int32_t k = 0; k < nsteps; ++k) {
    uint64_t step = (uint64_t)(first_step + k);
    if (s->m.integrator == ORC_RK4) rk4_step(s, spins, step);
    else heun_step(s, spins, step);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* observables                                                               */
/* ------------------------------------------------------------------------ */

int orc_energies(orc_sim *s, const double *spins, double t, double *e_terms) {
  const int64_t n = s->n;
  for (int tt = 0; tt < s->nt; ++tt) {
    const orc_term *tm = &s->terms[tt];
    double e = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      const double *sp = spins + 3 * i;
      const int b = (int)(i % s->m.nb);
      double f[3];
      switch (tm->kind) {
        case ORC_TERM_EXCHANGE:
          /* -1/2 sum s.h (sparse_interaction.cc:86-100) */
          term_field(s, tt, spins, i, t, f);
          e += -(sp[0] * f[0] + sp[1] * f[1] + sp[2] * f[2]);
          break;
        case ORC_TERM_UNIAXIAL: {
          /* uniaxial_anisotropy.cc:126-133 */
          const double *a = tm->axis + 3 * b;
          double dot = (a[0] * sp[0] + a[1] * sp[1] + a[2] * sp[2]);
          e += (-tm->K[b] * pow(dot, tm->order));
          break;
        }
        case ORC_TERM_CUBIC: {
          /* cubic_anisotropy.cc:135-156 */
          const double *u = tm->axis + 9 * b, *v = u + 3, *w = u + 6;
          double Su = sp[0] * u[0] + sp[1] * u[1] + sp[2] * u[2];
          double Sv = sp[0] * v[0] + sp[1] * v[1] + sp[2] * v[2];
          double Sw = sp[0] * w[0] + sp[1] * w[1] + sp[2] * w[2];
          double Su2 = Su * Su, Sv2 = Sv * Sv, Sw2 = Sw * Sw;
          if (tm->order == 1) e += -tm->K[b] * (Su2 * Sv2 + Sv2 * Sw2 + Sw2 * Su2);
          else e += -tm->K[b] * (Su2 * Sv2 * Sw2);
          break;
        }
        case ORC_TERM_DIPOLE:
          /* -1/2 sum s.h (cuda_dipole_fft.cu:156-167) */
          term_field(s, tt, spins, i, t, f);
          e += -(sp[0] * f[0] + sp[1] * f[1] + sp[2] * f[2]);
          break;
        default:
          /* applied_field.cc:150-155, zeeman.cc:82-87 */
          term_field(s, tt, spins, i, t, f);
          e += -(sp[0] * f[0] + sp[1] * f[1] + sp[2] * f[2]);
          break;
      }
    }
    if (tm->kind == ORC_TERM_EXCHANGE || tm->kind == ORC_TERM_DIPOLE) e = 0.5 * e;
    e_terms[tt] = e;
  }
  return 0;
}

/* magnetisation.cc:77-104 (normalised by the summed moments) */
int orc_magnetisation(const orc_sim *s, const double *spins, double *m4) {
  double mx = 0.0, my = 0.0, mz = 0.0, ms = 0.0;
  for (int64_t i = 0; i < s->n; ++i) {
    mx += spins[3 * i] * s->mus[i];
    my += spins[3 * i + 1] * s->mus[i];
    mz += spins[3 * i + 2] * s->mus[i];
    ms += s->mus[i];
  }
  m4[0] = mx / ms;
  m4[1] = my / ms;
  m4[2] = mz / ms;
  m4[3] = sqrt(mx * mx + my * my + mz * mz) / ms;
  return 0;
}

/* src/jams/monitors/topological_charge_geometrical_def.cc:159-181: each
   elementary triangle (i, j, k) taken counter-clockwise contributes
   2 atan2(s_i . (s_j x s_k), 1 + s_i.s_j + s_i.s_k + s_j.s_k); the sum is
   divided by 4 pi.  On the triangular lattice with a1 = (1, 0), a2 = (1/2,
   sqrt(3)/2) the triangles are (c, c + a1, c + a2) and (c + a1, c + a1 + a2,
   c + a2) for every cell c. */
static double tri_charge(const double *a, const double *b, const double *c) {
  double bxc[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
  double triple = a[0] * bxc[0] + a[1] * bxc[1] + a[2] * bxc[2];
  double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  double ac = a[0] * c[0] + a[1] * c[1] + a[2] * c[2];
  double bc = b[0] * c[0] + b[1] * c[1] + b[2] * c[2];
  double denominator = 1 + ab + ac + bc;
  return 2.0 * atan2(triple, denominator);
}

double orc_topological_charge_triangular(const double *spins, int32_t L1, int32_t L2) {
  double sum = 0.0;
  for (int64_t i = 0; i < L1; ++i)
    for (int64_t j = 0; j < L2; ++j) {
      int64_t ip = (i + 1) % L1, jp = (j + 1) % L2;
      const double *s00 = spins + 3 * (i * L2 + j);
      const double *s10 = spins + 3 * (ip * L2 + j);
      const double *s01 = spins + 3 * (i * L2 + jp);
      const double *s11 = spins + 3 * (ip * L2 + jp);
      sum += tri_charge(s00, s10, s01);
      sum += tri_charge(s10, s11, s01);
    }
  return sum / (4.0 * 3.14159265358979323846264338327950288);
}
