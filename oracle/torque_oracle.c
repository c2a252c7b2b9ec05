/*
 * torque_oracle.c -- CPU restatement of Torque's block-sparse contraction path.
 *
 * TEST INFRASTRUCTURE ONLY (see torque_oracle.h).  Plain C99, no dependencies,
 * builds with gcc on x86_64 and aarch64 alike.
 */
#include "torque_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXR 32

/* Free legs of a tensor in ascending order (arma shed_rows keeps the order of
 * the remaining rows: src/tensor/block_sparse.cpp:187-192). */
static int free_legs(int rank, int nc, const int64_t *legs, int *fl) {
  int n = 0;
  for (int l = 0; l < rank; l++) {
    int c = 0;
    for (int k = 0; k < nc; k++) c |= (legs[k] == l);
    if (!c) fl[n++] = l;
  }
  return n;
}

/* The overlap test of block_in_range (src/tensor/block_sparse.cpp:42-60). */
static int overlaps(const orc_bs *A, const orc_bs *B, int nc, const int64_t *al,
                    const int64_t *bl, int64_t i, int64_t j) {
  const int64_t *ab = A->begin + i * A->rank, *ae = A->end + i * A->rank;
  const int64_t *bb = B->begin + j * B->rank, *be = B->end + j * B->rank;
  for (int k = 0; k < nc; k++) {
    int64_t lo = ab[al[k]] > bb[bl[k]] ? ab[al[k]] : bb[bl[k]];
    int64_t hi = ae[al[k]] < be[bl[k]] ? ae[al[k]] : be[bl[k]];
    if (lo > hi) return 0;
  }
  return 1;
}

int64_t orc_match(const orc_bs *A, const orc_bs *B, int32_t nc,
                  const int64_t *a_legs, const int64_t *b_legs,
                  int64_t *pa, int64_t *pb, int64_t cap) {
  int64_t n = 0;
  for (int64_t i = 0; i < A->n_blocks; i++)
    for (int64_t j = 0; j < B->n_blocks; j++)
      if (overlaps(A, B, nc, a_legs, b_legs, i, j)) {
        if (pa) {
          if (n >= cap) return -1;
          pa[n] = i;
          pb[n] = j;
        }
        n++;
      }
  return n;
}

void orc_pair_boxes(const orc_bs *A, const orc_bs *B, int32_t nc,
                    const int64_t *al, const int64_t *bl, int64_t i, int64_t j,
                    int64_t *out_begin, int64_t *out_end, int64_t *con_begin,
                    int64_t *con_end, int64_t *a_sub_begin, int64_t *a_sub_end,
                    int64_t *b_sub_begin, int64_t *b_sub_end) {
  const int64_t *ab = A->begin + i * A->rank, *ae = A->end + i * A->rank;
  const int64_t *bb = B->begin + j * B->rank, *be = B->end + j * B->rank;
  int fa[MAXR], fb[MAXR];
  int nfa = free_legs(A->rank, nc, al, fa);
  int nfb = free_legs(B->rank, nc, bl, fb);
  int64_t cb[MAXR], ce[MAXR];
  for (int k = 0; k < nc; k++) {
    cb[k] = ab[al[k]] > bb[bl[k]] ? ab[al[k]] : bb[bl[k]];
    ce[k] = ae[al[k]] < be[bl[k]] ? ae[al[k]] : be[bl[k]];
  }
  if (out_begin)
    for (int q = 0; q < nfa + nfb; q++)
      out_begin[q] = q < nfa ? ab[fa[q]] : bb[fb[q - nfa]];
  if (out_end)
    for (int q = 0; q < nfa + nfb; q++)
      out_end[q] = q < nfa ? ae[fa[q]] : be[fb[q - nfa]];
  if (con_begin) memcpy(con_begin, cb, sizeof(int64_t) * nc);
  if (con_end) memcpy(con_end, ce, sizeof(int64_t) * nc);
  /* A/B sub-boxes: the block's own box with the contracted legs replaced by the
   * intersection (block_sparse.cpp:83-106, :130-148). */
  if (a_sub_begin) {
    memcpy(a_sub_begin, ab, sizeof(int64_t) * A->rank);
    for (int k = 0; k < nc; k++) a_sub_begin[al[k]] = cb[k];
  }
  if (a_sub_end) {
    memcpy(a_sub_end, ae, sizeof(int64_t) * A->rank);
    for (int k = 0; k < nc; k++) a_sub_end[al[k]] = ce[k];
  }
  if (b_sub_begin) {
    memcpy(b_sub_begin, bb, sizeof(int64_t) * B->rank);
    for (int k = 0; k < nc; k++) b_sub_begin[bl[k]] = cb[k];
  }
  if (b_sub_end) {
    memcpy(b_sub_end, be, sizeof(int64_t) * B->rank);
    for (int k = 0; k < nc; k++) b_sub_end[bl[k]] = ce[k];
  }
}

/* Neumaier-compensated accumulator. */
typedef struct { double s, c; } ksum;
static inline void kadd(ksum *k, double x) {
  double t = k->s + x;
  if ((k->s >= 0 ? k->s : -k->s) >= (x >= 0 ? x : -x))
    k->c += (k->s - t) + x;
  else
    k->c += (x - t) + k->s;
  k->s = t;
}

/* Number of values a tensor holds: the end of its furthest block. */
static int64_t n_values(const orc_bs *T) {
  int64_t n = 0;
  for (int64_t b = 0; b < T->n_blocks; b++) {
    int64_t e = T->offsets[b], c = 1;
    for (int l = 0; l < T->rank; l++) c *= T->end[b * T->rank + l] - T->begin[b * T->rank + l] + 1;
    if (e + c > n) n = e + c;
  }
  return n;
}

static int64_t max_of(const int64_t *v, int64_t n) {
  int64_t m = 0;
  for (int64_t i = 0; i < n; i++) if (v[i] > m) m = v[i];
  return m;
}

int32_t orc_pair_values(const orc_bs *A, const orc_bs *B, int32_t nc,
                        const int64_t *al, const int64_t *bl, int64_t i,
                        int64_t j, int64_t j_block, int32_t mode, double *out) {
  int fa[MAXR], fb[MAXR];
  int nfa = free_legs(A->rank, nc, al, fa);
  int nfb = free_legs(B->rank, nc, bl, fb);
  int64_t cb[MAXR], ce[MAXR], asb[MAXR], bsb[MAXR];
  orc_pair_boxes(A, B, nc, al, bl, i, j, NULL, NULL, cb, ce, asb, NULL, bsb,
                 NULL);
  const int64_t *ab = A->begin + i * A->rank, *bb = B->begin + j * B->rank;
  const int64_t *ae = A->end + i * A->rank, *be = B->end + j * B->rank;
  /* Base offsets use each block's own strides in every mode
   * (block_sparse.h:516-525). */
  const int64_t *sa_base = A->strides + i * A->rank;
  const int64_t *sb_base = B->strides + j * B->rank;
  int64_t base_a = A->offsets[i], base_b = B->offsets[j];
  for (int l = 0; l < A->rank; l++) base_a += (asb[l] - ab[l]) * sa_base[l];
  for (int l = 0; l < B->rank; l++) base_b += (bsb[l] - bb[l]) * sb_base[l];
  /* Element strides: own strides, or the reference's column j_block. */
  const int64_t *sa = sa_base, *sb = sb_base;
  if (mode == 2) {
    if (j_block >= A->n_blocks || j_block >= B->n_blocks) return ORC_ERR_RANGE;
    sa = A->strides + j_block * A->rank;
    sb = B->strides + j_block * B->rank;
  }
  int64_t md[MAXR], nd[MAXR], kd[MAXR];
  int64_t m = 1, n = 1, K = 1;
  for (int q = 0; q < nfa; q++) { md[q] = ae[fa[q]] - ab[fa[q]] + 1; m *= md[q]; }
  for (int q = 0; q < nfb; q++) { nd[q] = be[fb[q]] - bb[fb[q]] + 1; n *= nd[q]; }
  for (int k = 0; k < nc; k++) { kd[k] = ce[k] - cb[k] + 1; K *= kd[k]; }
  /* Address tables of A rows, B rows and the contracted columns. */
  int64_t *ra = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m ? m : 1));
  int64_t *rb = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
  int64_t *ka = (int64_t *)malloc(sizeof(int64_t) * (size_t)(K ? K : 1));
  int64_t *kb = (int64_t *)malloc(sizeof(int64_t) * (size_t)(K ? K : 1));
  for (int64_t r = 0; r < m; r++) {
    int64_t t = r, a = 0;
    for (int q = 0; q < nfa; q++) { a += (t % md[q]) * sa[fa[q]]; t /= md[q]; }
    ra[r] = a;
  }
  for (int64_t r = 0; r < n; r++) {
    int64_t t = r, a = 0;
    for (int q = 0; q < nfb; q++) { a += (t % nd[q]) * sb[fb[q]]; t /= nd[q]; }
    rb[r] = a;
  }
  for (int64_t c = 0; c < K; c++) {
    int64_t t = c, x = 0, y = 0;
    for (int k = 0; k < nc; k++) {
      int64_t v = t % kd[k];
      t /= kd[k];
      x += v * sa[al[k]];
      y += v * sb[bl[k]];
    }
    ka[c] = x;
    kb[c] = y;
  }
  if (mode == 2 && m > 0 && n > 0 && K > 0 &&
      (base_a + max_of(ra, m) + max_of(ka, K) >= n_values(A) ||
       base_b + max_of(rb, n) + max_of(kb, K) >= n_values(B))) {
    free(ra); free(rb); free(ka); free(kb);
    return ORC_ERR_READ;
  }
  const double *pa = A->data + base_a, *pb = B->data + base_b;
  for (int64_t c = 0; c < n; c++)
    for (int64_t r = 0; r < m; r++) {
      if (mode == 0) {
        ksum s = {0.0, 0.0};
        for (int64_t k = 0; k < K; k++) kadd(&s, pa[ra[r] + ka[k]] * pb[rb[c] + kb[k]]);
        out[r + c * m] = s.s + s.c;
      } else {
        double s = 0.0;
        for (int64_t k = 0; k < K; k++) s += pa[ra[r] + ka[k]] * pb[rb[c] + kb[k]];
        out[r + c * m] = s;
      }
    }
  free(ra); free(rb); free(ka); free(kb);
  return ORC_OK;
}

/* Gather the sub-box of block b (rows over free legs fl, columns over the
 * contracted legs cl restricted to [cb, ce]) into a contiguous row-major
 * rows x K matrix, as sort_into_matrix does. */
static void gather_rep(const orc_bs *T, int64_t b, int nf, const int *fl, int nc,
                       const int64_t *cl, const int64_t *cb, const int64_t *ce, double *out,
                       int64_t *rows_out, int64_t *k_out) {
  const int64_t *bb = T->begin + b * T->rank, *be = T->end + b * T->rank;
  const int64_t *st = T->strides + b * T->rank;
  int64_t base = T->offsets[b], rows = 1, K = 1, rd[MAXR], kd[MAXR];
  for (int q = 0; q < nf; q++) { rd[q] = be[fl[q]] - bb[fl[q]] + 1; rows *= rd[q]; }
  for (int k = 0; k < nc; k++) {
    kd[k] = ce[k] - cb[k] + 1;
    K *= kd[k];
    base += (cb[k] - bb[cl[k]]) * st[cl[k]];
  }
  for (int64_t r = 0; r < rows; r++) {
    int64_t t = r, ra = base;
    for (int q = 0; q < nf; q++) { ra += (t % rd[q]) * st[fl[q]]; t /= rd[q]; }
    for (int64_t c = 0; c < K; c++) {
      int64_t u = c, a = ra;
      for (int k = 0; k < nc; k++) { a += (u % kd[k]) * st[cl[k]]; u /= kd[k]; }
      out[r * K + c] = T->data[a];
    }
  }
  *rows_out = rows;
  *k_out = K;
}

int32_t orc_pairs_baseline(const orc_bs *A, const orc_bs *B, int32_t nc, const int64_t *al,
                           const int64_t *bl, int64_t n, const int64_t *pa, const int64_t *pb,
                           const int64_t *out_offsets, double *out) {
  int fa[MAXR], fb[MAXR];
  const int nfa = free_legs(A->rank, nc, al, fa);
  const int nfb = free_legs(B->rank, nc, bl, fb);
  int32_t threads = 1;
#ifdef _OPENMP
#pragma omp parallel
  {
#pragma omp single
    threads = omp_get_num_threads();
  }
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t q = 0; q < n; q++) {
    int64_t cb[MAXR], ce[MAXR], m, n_, K, K2;
    orc_pair_boxes(A, B, nc, al, bl, pa[q], pb[q], NULL, NULL, cb, ce, NULL, NULL, NULL, NULL);
    int64_t mm = 1, nn = 1, kk = 1;
    for (int x = 0; x < nfa; x++) mm *= A->end[pa[q] * A->rank + fa[x]] - A->begin[pa[q] * A->rank + fa[x]] + 1;
    for (int x = 0; x < nfb; x++) nn *= B->end[pb[q] * B->rank + fb[x]] - B->begin[pb[q] * B->rank + fb[x]] + 1;
    for (int k = 0; k < nc; k++) kk *= ce[k] - cb[k] + 1;
    double *ra = (double *)malloc(sizeof(double) * (size_t)(mm * kk));
    double *rb = (double *)malloc(sizeof(double) * (size_t)(nn * kk));
    gather_rep(A, pa[q], nfa, fa, nc, al, cb, ce, ra, &m, &K);
    gather_rep(B, pb[q], nfb, fb, nc, bl, cb, ce, rb, &n_, &K2);
    double *c = out + out_offsets[q];
    for (int64_t j = 0; j < n_; j++)
      for (int64_t i = 0; i < m; i++) {
        const double *x = ra + i * K, *y = rb + j * K;
        double s = 0.0;
        for (int64_t k = 0; k < K; k++) s += x[k] * y[k];
        c[i + j * m] = s;
      }
    free(ra);
    free(rb);
  }
  return threads;
}

int64_t orc_contract_size(const orc_bs *A, const orc_bs *B, int32_t nc,
                          const int64_t *al, const int64_t *bl) {
  int fa[MAXR], fb[MAXR];
  int nfa = free_legs(A->rank, nc, al, fa);
  int nfb = free_legs(B->rank, nc, bl, fb);
  if (nfa + nfb == 0) return 1;
  int64_t total = 0;
  for (int64_t i = 0; i < A->n_blocks; i++) {
    int64_t m = 1;
    for (int q = 0; q < nfa; q++)
      m *= A->end[i * A->rank + fa[q]] - A->begin[i * A->rank + fa[q]] + 1;
    for (int64_t j = 0; j < B->n_blocks; j++)
      if (overlaps(A, B, nc, al, bl, i, j)) {
        int64_t n = 1;
        for (int q = 0; q < nfb; q++)
          n *= B->end[j * B->rank + fb[q]] - B->begin[j * B->rank + fb[q]] + 1;
        total += m * n;
      }
  }
  return total;
}

int32_t orc_contract(const orc_bs *A, const orc_bs *B, int32_t nc,
                     const int64_t *al, const int64_t *bl, int32_t mode,
                     int64_t *out_begin, int64_t *out_end, int64_t *out_offsets,
                     double *out_data) {
  int fa[MAXR], fb[MAXR];
  int nfa = free_legs(A->rank, nc, al, fa);
  int nfb = free_legs(B->rank, nc, bl, fb);
  int ro = nfa + nfb;
  int64_t p = 0, off = 0;
  if (ro == 0) out_data[0] = 0.0;
  for (int64_t i = 0; i < A->n_blocks; i++) {
    int64_t jb = 0;
    for (int64_t j = 0; j < B->n_blocks; j++) {
      if (!overlaps(A, B, nc, al, bl, i, j)) continue;
      if (ro == 0) {
        /* Rank-0 result: the scalar loop of block_sparse.h:553-579 uses the
         * pair's own strides (no j_block indexing there). */
        double v;
        int32_t st = orc_pair_values(A, B, nc, al, bl, i, j, jb, mode == 2 ? 1 : mode, &v);
        if (st) return st;
        out_data[0] += v;
      } else {
        int64_t ob[MAXR], oe[MAXR], cnt = 1;
        orc_pair_boxes(A, B, nc, al, bl, i, j, ob, oe, NULL, NULL, NULL, NULL,
                       NULL, NULL);
        for (int q = 0; q < ro; q++) cnt *= oe[q] - ob[q] + 1;
        if (out_begin) memcpy(out_begin + p * ro, ob, sizeof(int64_t) * ro);
        if (out_end) memcpy(out_end + p * ro, oe, sizeof(int64_t) * ro);
        if (out_offsets) out_offsets[p] = off;
        if (out_data) {
          int32_t st = orc_pair_values(A, B, nc, al, bl, i, j, jb, mode, out_data + off);
          if (st) return st;
        }
        off += cnt;
      }
      p++;
      jb++;
    }
  }
  return ORC_OK;
}

static int in_block(const orc_bs *T, int64_t b, const int64_t *idx) {
  for (int l = 0; l < T->rank; l++)
    if (idx[l] < T->begin[b * T->rank + l] || idx[l] > T->end[b * T->rank + l])
      return 0;
  return 1;
}

double orc_query(const orc_bs *T, const int64_t *idx) {
  double s = 0.0;
  if (T->rank == 0) return T->n_blocks ? 0.0 : T->data[0];
  for (int64_t b = 0; b < T->n_blocks; b++) {
    if (!in_block(T, b, idx)) continue;
    int64_t a = T->offsets[b];
    for (int l = 0; l < T->rank; l++)
      a += (idx[l] - T->begin[b * T->rank + l]) * T->strides[b * T->rank + l];
    s += T->data[a];
  }
  return s;
}

void orc_densify(const orc_bs *T, double *dense) {
  int64_t total = 1, gs[MAXR];
  for (int l = 0; l < T->rank; l++) { gs[l] = total; total *= T->dimension[l]; }
  memset(dense, 0, sizeof(double) * (size_t)total);
  for (int64_t b = 0; b < T->n_blocks; b++) {
    int64_t dims[MAXR], cnt = 1;
    for (int l = 0; l < T->rank; l++) {
      dims[l] = T->end[b * T->rank + l] - T->begin[b * T->rank + l] + 1;
      cnt *= dims[l];
    }
    for (int64_t e = 0; e < cnt; e++) {
      int64_t t = e, src = T->offsets[b], dst = 0;
      for (int l = 0; l < T->rank; l++) {
        int64_t x = t % dims[l];
        t /= dims[l];
        src += x * T->strides[b * T->rank + l];
        dst += (x + T->begin[b * T->rank + l]) * gs[l];
      }
      dense[dst] += T->data[src];
    }
  }
}

void orc_hard_transpose(const orc_bs *T, const int64_t *perm, double *out) {
  int r = T->rank;
  for (int64_t b = 0; b < T->n_blocks; b++) {
    int64_t dims[MAXR], nd[MAXR], ns[MAXR], cnt = 1;
    for (int l = 0; l < r; l++)
      dims[l] = T->end[b * r + l] - T->begin[b * r + l] + 1;
    for (int l = 0; l < r; l++) { nd[l] = dims[perm[l]]; }
    for (int l = 0; l < r; l++) { ns[l] = cnt; cnt *= nd[l]; }
    /* new leg l holds old leg perm[l] (block_sparse.h:615-643) */
    for (int64_t e = 0; e < cnt; e++) {
      int64_t t = e, src = T->offsets[b];
      int64_t x[MAXR];
      for (int l = 0; l < r; l++) { x[l] = t % dims[l]; t /= dims[l]; }
      for (int l = 0; l < r; l++) src += x[l] * T->strides[b * r + l];
      int64_t dst = 0;
      for (int l = 0; l < r; l++) dst += x[perm[l]] * ns[l];
      out[T->offsets[b] + dst] = T->data[src];
    }
  }
}

void orc_nest_sum(const int64_t *x, int64_t n, int64_t *out) {
  int64_t t = 0;
  for (int64_t i = 0; i < n; i++) { out[i] = t; t += x[i]; }
}
