/*
 * ls_oracle.c -- CPU restatement of lattice-symmetries' exact-diagonalization hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library is compared
 * against, and the timed CPU baseline of bench.py.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU legs load it; the product library never links or calls it.
 *
 * What is restated (reference paths relative to the lattice-symmetries source tree):
 *   - orbit scan `state_info`        kernels/generator.cpp:10-166   (lane/chunk order emulated)
 *   - orbit scan `is_representative` kernels/generator.cpp:168-272  (early exit emulated)
 *   - spin-inversion / kernel choice kernels/kernels.c:96-98, :173-187
 *   - enumeration                    chapel/src/StatesEnumeration.chpl:29-73, :242-346
 *   - combinadics                    haskell/src/LatticeSymmetries/Basis.hs:487-550
 *   - state index (prefix table)     kernels/indexing.c:45-117, :196-215, :273-325
 *   - term generation                kernels/reference.c:67-134 = BatchedOperator.chpl:14-83
 *   - projection + rescale           chapel/src/BatchedOperator.chpl:139-253
 *   - accumulate (scatter)           chapel/src/DistributedMatrixVector.chpl:34-143, :1045-1058
 *
 * Two orbit-scan implementations exist: the checker applies each permutation bit by bit
 * (bit i of g.x = bit perm[g][i] of x, Benes.hs:338-345), independent of any Benes network;
 * the baseline applies the batched Benes network like the reference's Halide kernels.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------------ */
/* Group description                                                                            */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
  int n_bits;              /* number of bits of a basis state */
  int n_elems;             /* |G| */
  int spin_inversion;      /* 0, +1, -1 */
  const int32_t *perms;    /* [n_elems][n_bits] */
  const double *chars_re;  /* [n_elems] */
  const double *chars_im;  /* [n_elems] */
  int depth;               /* Benes network (baseline path); masks [depth][n_elems] */
  const uint64_t *masks;
  const uint64_t *shifts;
} lso_group;

static inline uint64_t flip_mask_of(int n) { return n == 0 ? 0 : (~(uint64_t)0) >> (64 - n); }

static inline uint64_t apply_perm(const lso_group *g, int e, uint64_t x) {
  const int32_t *p = g->perms + (int64_t)e * g->n_bits;
  uint64_t y = 0;
  for (int i = 0; i < g->n_bits; ++i) y |= ((x >> p[i]) & 1u) << i;
  return y;
}

static inline uint64_t apply_benes(const lso_group *g, int e, uint64_t x) {
  for (int k = 0; k < g->depth; ++k) {
    uint64_t m = g->masks[(int64_t)k * g->n_elems + e];
    unsigned d = (unsigned)g->shifts[k];
    uint64_t y = ((x >> d) ^ x) & m;
    x = x ^ y ^ (y << d);
  }
  return x;
}

static inline uint64_t image(const lso_group *g, int e, uint64_t x, int use_benes) {
  return use_benes ? apply_benes(g, e, x) : apply_perm(g, e, x);
}

/* Images of the W consecutive elements e0 .. e0 + W - 1 (W <= LSO_MAX_W): the reference's Halide
 * kernels evaluate a chunk of W group elements as one vector (generator.cpp:80, :155-164); the
 * lane loop below is written so that the compiler vectorises it the same way (the masks of one
 * stage are contiguous over the elements, kernels.c:157-167). */
#define LSO_MAX_W 16
static inline void images_chunk_fixed(const lso_group *g, int e0, uint64_t x, uint64_t *out, const int W) {
  uint64_t v[LSO_MAX_W];
  for (int j = 0; j < W; ++j) v[j] = x;
  for (int k = 0; k < g->depth; ++k) {
    const uint64_t *m = g->masks + (int64_t)k * g->n_elems + e0;
    const unsigned d = (unsigned)g->shifts[k];
    for (int j = 0; j < W; ++j) {
      const uint64_t y = ((v[j] >> d) ^ v[j]) & m[j];
      v[j] = v[j] ^ y ^ (y << d);
    }
  }
  for (int j = 0; j < W; ++j) out[j] = v[j];
}

static inline void images_chunk(const lso_group *g, int e0, int W, uint64_t x, int use_benes, uint64_t *out) {
  if (!use_benes) {
    for (int j = 0; j < W; ++j) out[j] = apply_perm(g, e0 + j, x);
    return;
  }
  /* constant lane counts of the reference's builds: fully unrolled and vectorised */
  if (W == 8) {
    images_chunk_fixed(g, e0, x, out, 8);
    return;
  }
  if (W == 4) {
    images_chunk_fixed(g, e0, x, out, 4);
    return;
  }
  uint64_t v[LSO_MAX_W];
  for (int j = 0; j < LSO_MAX_W; ++j) v[j] = x;
  for (int k = 0; k < g->depth; ++k) {
    const uint64_t *m = g->masks + (int64_t)k * g->n_elems + e0;
    const unsigned d = (unsigned)g->shifts[k];
    for (int j = 0; j < W; ++j) {
      const uint64_t y = ((v[j] >> d) ^ v[j]) & m[j];
      v[j] = v[j] ^ y ^ (y << d);
    }
  }
  for (int j = 0; j < W; ++j) out[j] = v[j];
}

/* ------------------------------------------------------------------------------------------ */
/* state_info: generator.cpp:10-166.                                                            */
/*   Per lane j < W: running (r, c, n) starting at (x, 1, 0); chunks m take element m*W + j.    */
/*   Lanes combine in order 0..W-1 (strict <, n summed); the tail elements follow in order.     */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
  uint64_t r;
  double cre, cim, n;
} si_acc;

static inline void si_step(si_acc *a, uint64_t x, uint64_t y, double cre, double cim) {
  if (y < a->r) {
    a->r = y;
    a->cre = cre;
    a->cim = cim;
  }
  if (y == x) a->n = a->n + cre;
}

static inline void si_elem(const lso_group *g, si_acc *a, uint64_t x, uint64_t y, int e) {
  double cre = g->chars_re[e], cim = g->chars_im[e];
  si_step(a, x, y, cre, cim);
  if (g->spin_inversion == 1) {
    si_step(a, x, y ^ flip_mask_of(g->n_bits), cre, cim);
  } else if (g->spin_inversion == -1) {
    si_step(a, x, y ^ flip_mask_of(g->n_bits), -cre, -cim);
  }
}

static si_acc state_info_one(const lso_group *g, int W, int use_benes, uint64_t x) {
  const int G = g->n_elems;
  const int nchunks = W <= LSO_MAX_W ? G / W : 0;
  si_acc lanes[LSO_MAX_W];
  uint64_t img[LSO_MAX_W];
  for (int j = 0; j < W && j < LSO_MAX_W; ++j) {
    lanes[j].r = x; lanes[j].cre = 1.0; lanes[j].cim = 0.0; lanes[j].n = 0.0;
  }
  /* chunk m: lane j takes element m * W + j; each lane sees its elements in chunk order */
  for (int m = 0; m < nchunks; ++m) {
    images_chunk(g, m * W, W, x, use_benes, img);
    for (int j = 0; j < W; ++j) si_elem(g, &lanes[j], x, img[j], m * W + j);
  }
  si_acc total = {x, 1.0, 0.0, 0.0};
  if (nchunks > 0) {
    total = lanes[0];
    for (int j = 1; j < W; ++j) {
      if (lanes[j].r < total.r) {
        total.r = lanes[j].r;
        total.cre = lanes[j].cre;
        total.cim = lanes[j].cim;
      }
      total.n = total.n + lanes[j].n;
    }
  }
  for (int e = nchunks * W; e < G; ++e) si_elem(g, &total, x, image(g, e, x, use_benes), e);
  return total;
}

void lso_state_info(const lso_group *g, int lane_width, int use_benes, int64_t count,
                    const uint64_t *xs, uint64_t *reps, double *chars /* 2*count */,
                    double *norms) {
  const int G = g->n_elems;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) {
    si_acc total = state_info_one(g, lane_width, use_benes, xs[i]);
    reps[i] = total.r;
    chars[2 * i] = total.cre;
    chars[2 * i + 1] = total.cim;
    norms[i] = sqrt(total.n / (double)(g->spin_inversion == 0 ? G : 2 * G));
  }
}

/* Exact stabiliser sum: |Stab| when every stabiliser character has real part exactly 1, else 0. */
static double exact_stabiliser_sum(const lso_group *g, int use_benes, uint64_t x) {
  const uint64_t flip = flip_mask_of(g->n_bits);
  int n = 0, trivial = 1;
  for (int e = 0; e < g->n_elems; ++e) {
    const uint64_t y = image(g, e, x, use_benes);
    if (y == x) {
      ++n;
      if (g->chars_re[e] != 1.0) trivial = 0;
    }
    if (g->spin_inversion != 0 && (y ^ flip) == x) {
      ++n;
      if ((double)g->spin_inversion * g->chars_re[e] != 1.0) trivial = 0;
    }
  }
  return trivial ? (double)n : 0.0;
}

/* ------------------------------------------------------------------------------------------ */
/* is_representative: generator.cpp:168-272 (chunked, early exit after the first chunk that    */
/* contains a smaller image; the tail is always added).                                         */
/* ------------------------------------------------------------------------------------------ */

static inline void ir_temp(const lso_group *g, uint64_t x, uint64_t y, int e, double *s, int *ge) {
  const double cre = g->chars_re[e];
  if (g->spin_inversion == 0) {
    *s = (double)(y == x) * cre;
    *ge = y >= x;
  } else {
    uint64_t yf = y ^ flip_mask_of(g->n_bits);
    double a = (double)(y == x), b = (double)(yf == x);
    *s = (g->spin_inversion == 1 ? a + b : a - b) * cre;
    *ge = (y >= x) && (yf >= x);
  }
}

static inline void is_rep_one(const lso_group *g, int W, int use_benes, uint64_t x, uint8_t *flag,
                              double *norm) {
  const int G = g->n_elems;
  const int nchunks = W <= LSO_MAX_W ? G / W : 0;
  uint64_t img[LSO_MAX_W];
  double sum = 0.0;
  int ok = 1;
  for (int m = 0; m < nchunks && ok; ++m) {
    double ls = 0.0;
    int lok = 1;
    images_chunk(g, m * W, W, x, use_benes, img);
    for (int j = 0; j < W; ++j) {
      double s;
      int ge;
      ir_temp(g, x, img[j], m * W + j, &s, &ge);
      ls = ls + s;
      lok = lok && ge;
    }
    sum = sum + ls;
    ok = ok && lok;
  }
  for (int e = nchunks * W; e < G; ++e) {
    double s;
    int ge;
    ir_temp(g, x, image(g, e, x, use_benes), e, &s, &ge);
    sum = sum + s;
    ok = ok && ge;
  }
  *norm = sum;
  *flag = (sum > 0) ? (uint8_t)ok : 0;
}

void lso_is_representative(const lso_group *g, int lane_width, int use_benes, int64_t count,
                           const uint64_t *xs, uint8_t *flags, double *norms) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) is_rep_one(g, lane_width, use_benes, xs[i], flags + i, norms + i);
}

/* Exact orbit data used by the checker where the reference's floating sums are exact:
 * representative, index of the first minimising element, and the stabiliser count when the
 * character is trivial on the stabiliser (0 otherwise). */
void lso_orbit_exact(const lso_group *g, int64_t count, const uint64_t *xs, uint64_t *reps,
                     int32_t *stab_count) {
  const uint64_t flip = flip_mask_of(g->n_bits);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) {
    uint64_t x = xs[i], best = x;
    int n = 0, trivial = 1;
    for (int e = 0; e < g->n_elems; ++e) {
      uint64_t y = apply_perm(g, e, x);
      for (int f = 0; f < (g->spin_inversion ? 2 : 1); ++f) {
        uint64_t z = f ? (y ^ flip) : y;
        double c = g->chars_re[e] * (f && g->spin_inversion == -1 ? -1.0 : 1.0);
        if (z < best) best = z;
        if (z == x) {
          ++n;
          if (c != 1.0) trivial = 0;
        }
      }
    }
    reps[i] = best;
    stab_count[i] = trivial ? n : 0;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Combinadics: Basis.hs:487-550.                                                               */
/* ------------------------------------------------------------------------------------------ */

static uint64_t binom_table[65][65];
static int binom_ready = 0;

static void binom_init(void) {
  if (binom_ready) return;
  memset(binom_table, 0, sizeof(binom_table));
  binom_table[0][0] = 1;
  for (int n = 1; n <= 64; ++n) {
    binom_table[n][0] = 1;
    for (int k = 1; k <= n; ++k) binom_table[n][k] = binom_table[n - 1][k - 1] + binom_table[n - 1][k];
  }
  binom_ready = 1;
}

/* binomial n k = 0 when n <= 0 or k > n (Basis.hs:506-509). */
static inline uint64_t binomial(int n, int k) {
  if (n <= 0 || k > n) return 0;
  return binom_table[n][k];
}

int64_t lso_fixed_hamming_state_to_index(uint64_t a) {
  binom_init();
  int64_t i = 0;
  for (int k = 1; a != 0; ++k) {
    int c = __builtin_ctzll(a);
    a &= a - 1;
    i += (int64_t)binomial(c, k);
  }
  return i;
}

uint64_t lso_fixed_hamming_index_to_state(int64_t index, int h) {
  binom_init();
  uint64_t state = 0;
  for (int i = h; i > 0; --i) {
    int c = i - 1;
    uint64_t contribution = binomial(c, i);
    while (c < 64) {
      uint64_t nc = binomial(c + 1, i);
      if ((int64_t)nc > index) break;
      ++c;
      contribution = nc;
    }
    state |= (uint64_t)1 << c;
    index -= (int64_t)contribution;
  }
  return state;
}

/* ------------------------------------------------------------------------------------------ */
/* Enumeration: StatesEnumeration.chpl:29-73 (Gosper step), :242-346.                           */
/* ------------------------------------------------------------------------------------------ */

static inline uint64_t next_fixed_hamming(uint64_t v) {
  uint64_t t = v | (v - 1);
  return (t + 1) | (((~t & (t + 1)) - 1) >> (__builtin_ctzll(v) + 1));
}

typedef struct {
  int particle_type;   /* 0 spin, 1 spinful fermion, 2 spinless fermion */
  int number_sites;
  int number_particles; /* -1 if not fixed */
  int number_up;        /* -1 if not fixed */
  int spin_inversion;
  int has_permutations;
  int hamming_fixed;
} lso_basis;

/* Projected spin enumeration over [lower, upper] (StatesEnumeration.chpl:242-268). */
int64_t lso_enumerate_projected(const lso_group *g, int lane_width, int use_benes, int hamming_fixed,
                                uint64_t lower, uint64_t upper, uint64_t *out, int64_t cap) {
  enum { B = 10240 }; /* kIsRepresentativeBatchSize, CommonParameters.chpl:5 */
  uint64_t *buf = (uint64_t *)malloc(B * sizeof(uint64_t));
  uint8_t *flags = (uint8_t *)malloc(B);
  double *norms = (double *)malloc(B * sizeof(double));
  int64_t written_total = 0;
  uint64_t v = lower;
  int done = (lower > upper);
  while (!done) {
    int n = 0;
    while (n < B) {
      buf[n++] = v;
      if (v == upper) {
        done = 1;
        break;
      }
      v = hamming_fixed ? next_fixed_hamming(v) : v + 1;
    }
    lso_is_representative(g, lane_width, use_benes, n, buf, flags, norms);
    for (int i = 0; i < n; ++i) {
      if (flags[i] && norms[i] > 0) {
        if (written_total < cap) out[written_total] = buf[i];
        ++written_total;
      }
    }
  }
  free(buf);
  free(flags);
  free(norms);
  return written_total;
}

/* Projected spin enumeration over [lower, upper] on all threads: the candidate range is split
 * into pieces by combinadic rank (StatesEnumeration.chpl:130-189 splits it among tasks the same
 * way), each piece walks its candidates in Gosper order (:29-32) and keeps a candidate iff
 * is_representative flags it and its floating norm is positive (:242-268); the pieces are joined
 * in order, so the output is sorted.  Returns the number of representatives (written up to cap). */
int64_t lso_enumerate_projected_par(const lso_group *g, int lane_width, int use_benes, int hamming_fixed,
                                    uint64_t lower, uint64_t upper, uint64_t *out, int64_t cap) {
  if (lower > upper) return 0;
  const int h = __builtin_popcountll(lower);
  const int64_t r0 = hamming_fixed ? lso_fixed_hamming_state_to_index(lower) : (int64_t)lower;
  const int64_t r1 = hamming_fixed ? lso_fixed_hamming_state_to_index(upper) : (int64_t)upper;
  const int64_t n = r1 - r0 + 1;
  int threads = 1;
#ifdef _OPENMP
  threads = omp_get_max_threads();
#endif
  int64_t pieces = (int64_t)threads * 64;
  if (pieces > n) pieces = n;
  uint64_t **bufs = (uint64_t **)calloc((size_t)pieces, sizeof(uint64_t *));
  int64_t *lens = (int64_t *)calloc((size_t)pieces, sizeof(int64_t));
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t p = 0; p < pieces; ++p) {
    const int64_t a = r0 + n * p / pieces, b = r0 + n * (p + 1) / pieces; /* ranks [a, b) */
    int64_t cap_p = 1024, len = 0;
    uint64_t *buf = (uint64_t *)malloc((size_t)cap_p * sizeof(uint64_t));
    uint64_t v = hamming_fixed ? lso_fixed_hamming_index_to_state(a, h) : (uint64_t)a;
    for (int64_t k = a; k < b; ++k) {
      uint8_t flag;
      double norm;
      is_rep_one(g, lane_width, use_benes, v, &flag, &norm);
      if (flag && norm > 0) {
        if (len == cap_p) {
          cap_p *= 2;
          buf = (uint64_t *)realloc(buf, (size_t)cap_p * sizeof(uint64_t));
        }
        buf[len++] = v;
      }
      if (k + 1 < b) v = hamming_fixed ? next_fixed_hamming(v) : v + 1;
    }
    bufs[p] = buf;
    lens[p] = len;
  }
  int64_t total = 0;
  for (int64_t p = 0; p < pieces; ++p) {
    for (int64_t k = 0; k < lens[p]; ++k, ++total)
      if (total < cap) out[total] = bufs[p][k];
    free(bufs[p]);
  }
  free(bufs);
  free(lens);
  return total;
}

/* Unprojected enumeration (StatesEnumeration.chpl:269-289): all states in [low, high] with
 * the Hamming weight of low (or all integers), with high clipped to high ^ mask under spin
 * inversion. */
int64_t lso_enumerate_unprojected(int number_sites, int spin_inversion, int hamming_fixed,
                                  uint64_t low, uint64_t high, uint64_t *out, int64_t cap) {
  if (spin_inversion != 0) {
    uint64_t mask = flip_mask_of(number_sites);
    uint64_t h2 = high ^ mask;
    if (h2 < high) high = h2;
  }
  int64_t n = 0;
  if (low > high) return 0;
  uint64_t v = low;
  while (1) {
    if (n < cap) out[n] = v;
    ++n;
    if (v == high) break;
    v = hamming_fixed ? next_fixed_hamming(v) : v + 1;
  }
  return n;
}

/* Spinful fermions with both N_up and N_down fixed (StatesEnumeration.chpl:290-326). */
int64_t lso_enumerate_spinful(int number_sites, uint64_t lower, uint64_t upper, uint64_t *out,
                              int64_t cap) {
  const uint64_t mask = flip_mask_of(number_sites);
  uint64_t minA = lower & mask, maxA = upper & mask;
  uint64_t minB = (lower >> number_sites) & mask, maxB = (upper >> number_sites) & mask;
  int64_t n = 0;
  uint64_t xb = minB;
  while (1) {
    uint64_t xa = minA;
    while (1) {
      if (n < cap) out[n] = (xb << number_sites) | xa;
      ++n;
      if (xa == maxA) break;
      xa = next_fixed_hamming(xa);
    }
    if (xb == maxB) break;
    xb = next_fixed_hamming(xb);
  }
  return n;
}

/* ------------------------------------------------------------------------------------------ */
/* State index: indexing.c:45-117 (offset table), :196-215 (search), :273-325 (kernel).         */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
  int64_t number_states;
  const uint64_t *reps;
  int number_bits; /* prefix bits actually used */
  int shift;
  int64_t range_size;
  int64_t number_offsets;
  int64_t *offsets;
} lso_index;

void lso_index_init(lso_index *c, const uint64_t *reps, int64_t n, int number_bits, int prefix_bits) {
  c->number_states = n;
  c->reps = reps;
  c->number_bits = prefix_bits > number_bits ? number_bits : prefix_bits;
  c->shift = number_bits - c->number_bits;
  c->range_size = 0;
  c->number_offsets = 0;
  c->offsets = NULL;
  if (c->number_bits > 0) {
    int64_t size = (int64_t)1 << c->number_bits;
    c->number_offsets = size + 1;
    c->offsets = (int64_t *)malloc((size_t)c->number_offsets * sizeof(int64_t));
    int64_t k = 0;
    for (int64_t i = 0; i < size; ++i) {
      c->offsets[i] = k;
      while (k != n && (reps[k] >> c->shift) == (uint64_t)i) ++k;
    }
    c->offsets[size] = k;
    int64_t maxr = 0;
    for (int64_t i = 0; i < size; ++i) {
      int64_t r = c->offsets[i + 1] - c->offsets[i];
      if (r > maxr) maxr = r;
    }
    for (int64_t i = 0; i < size; ++i)
      if (c->offsets[i] > n - maxr) c->offsets[i] = n - maxr;
    c->range_size = maxr;
  }
}

void lso_index_free(lso_index *c) {
  free(c->offsets);
  c->offsets = NULL;
}

static inline int64_t lso_index_one(const lso_index *c, uint64_t needle) {
  int64_t start = c->offsets[needle >> c->shift];
  const uint64_t *base = c->reps + start;
  int64_t n = c->range_size;
  if (n == 0) return -1;
  while (n > 1) {
    int64_t half = n / 2;
    n -= half;
    base = (base[half] < needle) ? base + half : base;
  }
  base += *base < needle;
  int64_t k = base - c->reps;
  return (k < c->number_states && *base == needle) ? k : -1;
}

/* Heap-allocated prefix index (built once per basis, as the reference keeps it in the basis'
 * kernel data, reference.c:184-193). */
lso_index *lso_index_create(const uint64_t *reps, int64_t n, int number_bits, int prefix_bits) {
  lso_index *c = (lso_index *)malloc(sizeof(lso_index));
  lso_index_init(c, reps, n, number_bits, prefix_bits);
  return c;
}

void lso_index_destroy(lso_index *c) {
  if (c == NULL) return;
  lso_index_free(c);
  free(c);
}

void lso_state_index(const lso_index *c, int64_t count, const uint64_t *xs, int64_t *out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) out[i] = lso_index_one(c, xs[i]);
}

/* Plain lower_bound search, independent of the prefix table. */
static inline int64_t bsearch_index(const uint64_t *reps, int64_t n, uint64_t needle) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (reps[mid] < needle) lo = mid + 1; else hi = mid;
  }
  return (lo < n && reps[lo] == needle) ? lo : -1;
}

/* ------------------------------------------------------------------------------------------ */
/* Matrix-vector product (scatter form of the reference).                                      */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
  int n;
  const double *v; /* complex128 [n] interleaved */
  const uint64_t *m, *l, *r, *x, *s;
} lso_terms;

/* mode bits */
#define LSO_COMPLEX 1     /* complex x, y and coefficients (extension); else the reference's real path */
#define LSO_BENES 2       /* orbit scan through the Benes network (baseline) */
#define LSO_PREFIX_INDEX 4 /* prefix-table index (baseline); else plain lower_bound */
#define LSO_ATOMIC 8      /* OpenMP over columns with atomic adds (baseline); else serial */
#define LSO_EXACT_NORMS 16 /* exact stabiliser sums for the generated states' norms */

typedef struct {
  int projection;       /* 0 none, 1 inversion only, 2 full */
  int spin_inversion;
  int n_bits;
  int state_index_identity;
} lso_projection;

/* Orbit scan with the reference's float order (W = 8 lanes) for the projected case; with
 * exact_norms the norm uses the exact stabiliser sum instead of the floating sum of characters. */
static inline void project(const lso_group *g, const lso_projection *pr, int use_benes, int exact_norms,
                           uint64_t beta, uint64_t *rep, double *cre, double *cim, double *norm) {
  if (pr->projection == 0) {
    *rep = beta; *cre = 1.0; *cim = 0.0; *norm = 1.0;
    return;
  }
  if (pr->projection == 1) {
    uint64_t inv = beta ^ flip_mask_of(pr->n_bits);
    if (inv < beta) {
      *rep = inv; *cre = (double)pr->spin_inversion; *cim = 0.0;
    } else {
      *rep = beta; *cre = 1.0; *cim = 0.0;
    }
    *norm = 1.0;
    return;
  }
  si_acc a = state_info_one(g, 8, use_benes, beta);
  const double denom = (double)(g->spin_inversion == 0 ? g->n_elems : 2 * g->n_elems);
  *rep = a.r;
  *cre = a.cre;
  *cim = a.cim;
  *norm = sqrt((exact_norms ? exact_stabiliser_sum(g, use_benes, beta) : a.n) / denom);
}

/* y = H x over the representatives (BatchedOperator.chpl:139-282 + DistributedMatrixVector.chpl
 * :34-143).  Columns alpha_j scatter into rows.  Returns 0, or -1 if a non-zero coefficient hit
 * a state outside the basis (the reference halts there, DistributedMatrixVector.chpl:133). */
int lso_matvec(const lso_group *g, const lso_projection *pr, int64_t D, const uint64_t *reps,
               const double *rep_norms, const lso_terms *off, const lso_terms *diag, int mode,
               const double *x, double *y, int64_t row_begin, int64_t row_end, int64_t *nnz_out) {
  int64_t nnz = 0;
  const int cplx = mode & LSO_COMPLEX;
  const int use_benes = (mode & LSO_BENES) != 0;
  const int exact_norms = (mode & LSO_EXACT_NORMS) != 0;
  lso_index idx;
  int use_prefix = (mode & LSO_PREFIX_INDEX) != 0;
  if (use_prefix) lso_index_init(&idx, reps, D, pr->n_bits, 22);
  int error = 0;
  const int64_t stride = cplx ? 2 : 1;
  if (row_begin < 0) row_begin = 0;
  if (row_end < 0 || row_end > D) row_end = D;
  memset(y, 0, (size_t)(D * stride) * sizeof(double));
  /* Diagonal: BatchedOperator.chpl:14-45 (real part of v in the reference's real path). */
  if (diag != NULL && diag->n > 0) {
#pragma omp parallel for schedule(static) if (mode & LSO_ATOMIC)
    for (int64_t i = row_begin; i < row_end; ++i) {
      const uint64_t a = reps[i];
      double accr = 0.0, acci = 0.0;
      /* A representative whose norm is zero spans no state of the sector: its row and column
       * of H are zero (the reference divides by such norms; see the matvec kernels). */
      if (pr->projection == 2 && rep_norms[i] == 0.0) continue;
      for (int t = 0; t < diag->n; ++t) {
        if ((a & diag->m[t]) == diag->r[t]) {
          int sign = 1 - 2 * (__builtin_popcountll(a & diag->s[t]) % 2);
          if (cplx) {
            double xr = sign * x[2 * i], xi = sign * x[2 * i + 1];
            accr += diag->v[2 * t] * xr - diag->v[2 * t + 1] * xi;
            acci += diag->v[2 * t] * xi + diag->v[2 * t + 1] * xr;
          } else {
            accr += diag->v[2 * t] * (sign * x[i]);
          }
        }
      }
      y[stride * i] = accr;
      if (cplx) y[2 * i + 1] = acci;
    }
  }
  if (off != NULL && off->n > 0) {
#pragma omp parallel for schedule(dynamic, 64) if (mode & LSO_ATOMIC) reduction(+ : nnz)
    for (int64_t j = row_begin; j < row_end; ++j) {
      const uint64_t a = reps[j];
      const double na = pr->projection == 2 ? rep_norms[j] : 1.0;
      if (na == 0.0) continue; /* zero-norm representative: zero column */
      for (int t = 0; t < off->n; ++t) {
        if ((a & off->m[t]) != off->r[t]) continue;
        const int sign = 1 - 2 * (__builtin_popcountll(a & off->s[t]) % 2);
        /* coefficient v * (sign * x_j), BatchedOperator.chpl:72-77 */
        double cr, ci;
        if (cplx) {
          double xr = sign * x[2 * j], xi = sign * x[2 * j + 1];
          cr = off->v[2 * t] * xr - off->v[2 * t + 1] * xi;
          ci = off->v[2 * t] * xi + off->v[2 * t + 1] * xr;
        } else {
          double f = sign * x[j];
          cr = off->v[2 * t] * f;
          ci = off->v[2 * t + 1] * f;
        }
        const uint64_t beta = a ^ off->x[t];
        uint64_t rep;
        double chr, chi, nb;
        project(g, pr, use_benes, exact_norms, beta, &rep, &chr, &chi, &nb);
        /* cs *= tempCoeffs * norms[k] / norms[alpha] (BatchedOperator.chpl:242-246) */
        double sr = cr * nb / na, si = ci * nb / na;
        double outr = chr * sr - chi * si, outi = chr * si + chi * sr;
        if (!cplx) {
          if (outr == 0.0) continue; /* DistributedMatrixVector.chpl:126-127 */
        } else if (outr == 0.0 && outi == 0.0) {
          continue;
        }
        int64_t i;
        if (pr->state_index_identity)
          i = (int64_t)rep;
        else
          i = use_prefix ? lso_index_one(&idx, rep) : bsearch_index(reps, D, rep);
        if (i < 0) {
#pragma omp atomic write
          error = 1;
          continue;
        }
        ++nnz;
        if (cplx) {
#pragma omp atomic
          y[2 * i] += outr;
#pragma omp atomic
          y[2 * i + 1] += outi;
        } else {
#pragma omp atomic
          y[i] += outr;
        }
      }
    }
  }
  if (use_prefix) lso_index_free(&idx);
  if (nnz_out) *nnz_out = nnz;
  return error ? -1 : 0;
}

/* One column of the scatter (the per-column body of lso_matvec with x = e_j): calls emit(row,
 * re, im) for the diagonal element and for every non-zero off-diagonal element; returns -1 if a
 * non-zero element hit a state outside the basis, else the number of off-diagonal elements. */
typedef struct {
  int64_t *rows;
  double *vals;
  int64_t n;
} lso_col_sink;

static int64_t scatter_column(const lso_group *g, const lso_projection *pr, int64_t D, const uint64_t *reps,
                              const lso_index *idx, const lso_terms *off, const lso_terms *diag, int mode,
                              int64_t j, double na, double xre, double xim, lso_col_sink *sink, double *y) {
  const int use_benes = (mode & LSO_BENES) != 0;
  const int exact_norms = (mode & LSO_EXACT_NORMS) != 0;
  const uint64_t a = reps[j];
  int64_t found = 0;
  if (pr->projection == 2 && na == 0.0) return 0; /* zero-norm representative: zero column */
  if (diag != NULL && diag->n > 0) {
    double accr = 0.0, acci = 0.0;
    for (int t = 0; t < diag->n; ++t) {
      if ((a & diag->m[t]) == diag->r[t]) {
        int sign = 1 - 2 * (__builtin_popcountll(a & diag->s[t]) % 2);
        accr += diag->v[2 * t] * (sign * xre) - diag->v[2 * t + 1] * (sign * xim);
        acci += diag->v[2 * t] * (sign * xim) + diag->v[2 * t + 1] * (sign * xre);
      }
    }
    if (sink) {
      sink->rows[sink->n] = j;
      sink->vals[2 * sink->n] = accr;
      sink->vals[2 * sink->n + 1] = acci;
      ++sink->n;
    } else {
#pragma omp atomic
      y[2 * j] += accr;
#pragma omp atomic
      y[2 * j + 1] += acci;
    }
  }
  if (off == NULL) return 0;
  for (int t = 0; t < off->n; ++t) {
    if ((a & off->m[t]) != off->r[t]) continue;
    const int sign = 1 - 2 * (__builtin_popcountll(a & off->s[t]) % 2);
    const double xr = sign * xre, xi = sign * xim;
    const double cr = off->v[2 * t] * xr - off->v[2 * t + 1] * xi;
    const double ci = off->v[2 * t] * xi + off->v[2 * t + 1] * xr;
    const uint64_t beta = a ^ off->x[t];
    uint64_t rep;
    double chr, chi, nb;
    project(g, pr, use_benes, exact_norms, beta, &rep, &chr, &chi, &nb);
    const double sr = cr * nb / na, si = ci * nb / na;
    const double outr = chr * sr - chi * si, outi = chr * si + chi * sr;
    if (outr == 0.0 && outi == 0.0) continue;
    int64_t i;
    if (pr->state_index_identity)
      i = (int64_t)rep;
    else
      i = idx != NULL ? lso_index_one(idx, rep) : bsearch_index(reps, D, rep);
    if (i < 0) return -1;
    ++found;
    if (sink) {
      sink->rows[sink->n] = i;
      sink->vals[2 * sink->n] = outr;
      sink->vals[2 * sink->n + 1] = outi;
      ++sink->n;
    } else {
#pragma omp atomic
      y[2 * i] += outr;
#pragma omp atomic
      y[2 * i + 1] += outi;
    }
  }
  return found;
}

/* Columns cols[0..ncols) of H (complex arithmetic), element by element: column c writes its
 * elements (the diagonal one first) to rows[c * stride + k] and the complex values to
 * vals[2 * (c * stride + k) + {0, 1}], k < counts[c], stride = off->n + 1; col_norms[c] is the
 * norm of representative cols[c].  Returns 0, or -1 if an element hit a state outside the basis. */
int lso_matvec_columns(const lso_group *g, const lso_projection *pr, int64_t D, const uint64_t *reps,
                       const lso_index *idx, const lso_terms *off, const lso_terms *diag, int mode, int64_t ncols,
                       const int64_t *cols, const double *col_norms, int64_t *rows, double *vals,
                       int64_t *counts) {
  const int64_t stride = (off != NULL ? off->n : 0) + 1;
  int error = 0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t c = 0; c < ncols; ++c) {
    lso_col_sink sink = {rows + c * stride, vals + 2 * c * stride, 0};
    const double na = pr->projection == 2 ? col_norms[c] : 1.0;
    if (scatter_column(g, pr, D, reps, idx, off, diag, mode, cols[c], na, 1.0, 0.0, &sink, NULL) < 0) {
#pragma omp atomic write
      error = 1;
    }
    counts[c] = sink.n;
  }
  return error ? -1 : 0;
}

/* The reference's scatter over a sample of columns (DistributedMatrixVector.chpl:91-143 with
 * BatchedOperator.chpl:139-253): y[i] += H[i, cols[c]] * x[c] with relaxed atomic adds, all
 * threads, complex x and y (y has D entries and is not cleared).  *nnz_out = off-diagonal
 * elements generated.  Returns 0, or -1 if an element hit a state outside the basis. */
int lso_matvec_sample(const lso_group *g, const lso_projection *pr, int64_t D, const uint64_t *reps,
                      const lso_index *idx, const lso_terms *off, const lso_terms *diag, int mode, int64_t ncols,
                      const int64_t *cols, const double *col_norms, const double *x, double *y,
                      int64_t *nnz_out) {
  int64_t nnz = 0;
  int error = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : nnz)
  for (int64_t c = 0; c < ncols; ++c) {
    const double na = pr->projection == 2 ? col_norms[c] : 1.0;
    const int64_t f = scatter_column(g, pr, D, reps, idx, off, diag, mode, cols[c], na, x[2 * c], x[2 * c + 1],
                                     NULL, y);
    if (f < 0) {
#pragma omp atomic write
      error = 1;
    } else {
      nnz += f;
    }
  }
  if (nnz_out) *nnz_out = nnz;
  return error ? -1 : 0;
}

int lso_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void lso_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
