/*
 * ammsb_oracle_graph.c -- the synthetic workloads' graphs and held-out /
 * test sets, restated for the oracle, and a whole iteration of the oracle
 * sampler on several host threads.
 *
 * TEST INFRASTRUCTURE ONLY.  The CPU legs of the benchmark (the CPU
 * baseline and the reference arm) build their inputs here, so that they
 * load no library of the product; tests/test_oracle_graph.py checks that
 * these graphs and splits equal the product's (ammsb_generate_graph,
 * ammsb_make_held_out) element for element.
 *
 * The generator: community sizes from a continuous Zipf(s) tail, floored
 * and clipped to [size_min, size_max]; 1 / 2 / 3 memberships per node with
 * probabilities p1 / p2 / rest; the size list rescaled to cover the
 * membership slots, shuffled (Fisher-Yates) and dealt to nodes;
 * round(d * s / 2) uniform member pairs per community of s members; then
 * background_frac of that many uniform pairs; self-loops dropped and
 * duplicates merged into a symmetric CSR with sorted rows.  Every draw is a
 * Philox block of the stream tag 9 (graph) or 10 (held-out).
 *
 * The split follows network.cc:503-614: held_out_size = ratio * E
 * (truncated), p = held_out_size / 2 links and p non-links for the
 * held-out set, then p links and p non-links for the test set, which
 * avoids the held-out pairs.
 */
#include "ammsb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define TAG_GRAPH 9u
#define TAG_HELD_OUT 10u

static uint64_t draw(uint32_t seed, uint32_t tag, uint32_t entity,
                     uint32_t step, uint64_t t) {
  return oracle_draw_u64(seed, 0, tag, entity, step, t);
}

static double u01_open(uint64_t x) {
  return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static uint64_t key_of(int32_t a, int32_t b) {
  uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
  return ((uint64_t)lo << 32) | hi;
}

/* Sorts keys ascending: least-significant-digit radix sort, 16-bit digits,
 * over the low `bits` bits. */
static int sort_keys(uint64_t *keys, size_t n, int bits) {
  uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
  size_t *count = (size_t *)malloc(sizeof(size_t) * 65536);
  if (!tmp || !count) {
    free(tmp);
    free(count);
    return -1;
  }
  uint64_t *src = keys, *dst = tmp;
  for (int shift = 0; shift < bits; shift += 16) {
    memset(count, 0, sizeof(size_t) * 65536);
    for (size_t i = 0; i < n; ++i) count[(src[i] >> shift) & 0xffffu]++;
    size_t run = 0;
    for (size_t d = 0; d < 65536; ++d) {
      size_t c = count[d];
      count[d] = run;
      run += c;
    }
    for (size_t i = 0; i < n; ++i) dst[count[(src[i] >> shift) & 0xffffu]++] = src[i];
    uint64_t *sw = src;
    src = dst;
    dst = sw;
  }
  if (src != keys) memcpy(keys, src, sizeof(uint64_t) * n);
  free(tmp);
  free(count);
  return 0;
}

/* Symmetric CSR with sorted rows from undirected pair keys. */
static int csr_from_pairs(int64_t n, const uint64_t *pairs, size_t np,
                          int64_t **row_ptr_out, int32_t **col_out) {
  uint64_t *dir = (uint64_t *)malloc(sizeof(uint64_t) * (2 * np + 1));
  if (!dir) return -1;
  size_t m = 0;
  for (size_t i = 0; i < np; ++i) {
    uint32_t a = (uint32_t)(pairs[i] >> 32), b = (uint32_t)pairs[i];
    if (a == b) continue;
    dir[m++] = ((uint64_t)a << 32) | b;
    dir[m++] = ((uint64_t)b << 32) | a;
  }
  int bits = 32;
  for (uint64_t v = (uint64_t)(n > 0 ? n - 1 : 0); v; v >>= 1) ++bits;
  if (sort_keys(dir, m, bits) != 0) {
    free(dir);
    return -1;
  }
  size_t u = 0;
  for (size_t i = 0; i < m; ++i)
    if (u == 0 || dir[i] != dir[u - 1]) dir[u++] = dir[i];
  int64_t *row_ptr = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (u ? u : 1));
  if (!row_ptr || !col) {
    free(dir);
    free(row_ptr);
    free(col);
    return -1;
  }
  for (size_t i = 0; i < u; ++i) {
    row_ptr[(dir[i] >> 32) + 1]++;
    col[i] = (int32_t)(uint32_t)dir[i];
  }
  for (int64_t v = 0; v < n; ++v) row_ptr[v + 1] += row_ptr[v];
  free(dir);
  *row_ptr_out = row_ptr;
  *col_out = col;
  return 0;
}

int oracle_generate_graph(const oracle_gen_params *p, int64_t **row_ptr_out,
                          int32_t **col_out) {
  if (!p || p->n < 2 || p->k_true < 1 || p->size_min < 1 ||
      p->size_max < p->size_min || p->zipf_s <= 1.0 || p->p1 < 0 || p->p2 < 0 ||
      p->p1 + p->p2 > 1.0 || p->intra_degree < 0 || p->background_frac < 0 ||
      p->n > INT32_MAX)
    return -1;
  const uint32_t seed = p->seed;
  const int64_t n = p->n, kc = p->k_true;
  int rc = -1;
  double *size = (double *)malloc(sizeof(double) * (size_t)kc);
  int64_t *moff = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  int32_t *slot = NULL, *member = NULL;
  int64_t *coff = NULL, *fill = NULL;
  uint64_t *pairs = NULL;
  if (!size || !moff) goto out;

  double size_sum = 0.0;
  for (int64_t c = 0; c < kc; ++c) {
    double u = u01_open(draw(seed, TAG_GRAPH, 0, 0, (uint64_t)c));
    double s = floor((double)p->size_min * pow(u, -1.0 / (p->zipf_s - 1.0)));
    if (s < (double)p->size_min) s = (double)p->size_min;
    if (s > (double)p->size_max) s = (double)p->size_max;
    size[c] = s;
    size_sum += s;
  }
  moff[0] = 0;
  for (int64_t v = 0; v < n; ++v) {
    double u = u01_open(draw(seed, TAG_GRAPH, 1, 0, (uint64_t)v));
    moff[v + 1] = moff[v] + (u < p->p1 ? 1 : (u < p->p1 + p->p2 ? 2 : 3));
  }
  const int64_t M = moff[n];
  /* slots: each community's rescaled size, topped up to M */
  int64_t n_slot = 0, cap_slot = M + kc + 16;
  slot = (int32_t *)malloc(sizeof(int32_t) * (size_t)cap_slot);
  if (!slot) goto out;
  for (int64_t c = 0; c < kc; ++c) {
    long long s = llround(size[c] * (double)M / size_sum);
    if (s < 1) s = 1;
    if (n_slot + s > cap_slot) {
      cap_slot = 2 * (n_slot + s);
      int32_t *grown = (int32_t *)realloc(slot, sizeof(int32_t) * (size_t)cap_slot);
      if (!grown) goto out;
      slot = grown;
    }
    for (long long i = 0; i < s; ++i) slot[n_slot++] = (int32_t)c;
  }
  for (uint64_t t = 0; n_slot < M; ++t)
    slot[n_slot++] = (int32_t)(draw(seed, TAG_GRAPH, 2, 1, t) % (uint64_t)kc);
  for (int64_t i = n_slot - 1; i > 0; --i) {
    int64_t j = (int64_t)(draw(seed, TAG_GRAPH, 2, 0, (uint64_t)i) % (uint64_t)(i + 1));
    int32_t x = slot[i];
    slot[i] = slot[j];
    slot[j] = x;
  }
  /* slot[0 .. M) are the memberships of nodes in order */
  coff = (int64_t *)calloc((size_t)kc + 1, sizeof(int64_t));
  if (!coff) goto out;
  for (int64_t q = 0; q < M; ++q) coff[slot[q] + 1]++;
  for (int64_t c = 0; c < kc; ++c) coff[c + 1] += coff[c];
  member = (int32_t *)malloc(sizeof(int32_t) * (size_t)(coff[kc] + 1));
  fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(kc + 1));
  if (!member || !fill) goto out;
  memcpy(fill, coff, sizeof(int64_t) * (size_t)kc);
  for (int64_t v = 0; v < n; ++v)
    for (int64_t q = moff[v]; q < moff[v + 1]; ++q) member[fill[slot[q]]++] = (int32_t)v;

  /* intra-community pairs, then background pairs */
  size_t np = 0, cap_pairs = 1024;
  pairs = (uint64_t *)malloc(sizeof(uint64_t) * cap_pairs);
  if (!pairs) goto out;
  uint64_t t = 0;
  for (int64_t c = 0; c < kc; ++c) {
    int64_t s = coff[c + 1] - coff[c];
    if (s < 2) continue;
    long long want = llround(p->intra_degree * (double)s / 2.0);
    for (long long q = 0; q < want; ++q, t += 2) {
      int32_t a = member[coff[c] + (int64_t)(draw(seed, TAG_GRAPH, 3, 0, t) % (uint64_t)s)];
      int32_t b = member[coff[c] + (int64_t)(draw(seed, TAG_GRAPH, 3, 0, t + 1) % (uint64_t)s)];
      if (a == b) continue;
      if (np == cap_pairs) {
        cap_pairs *= 2;
        uint64_t *grown = (uint64_t *)realloc(pairs, sizeof(uint64_t) * cap_pairs);
        if (!grown) goto out;
        pairs = grown;
      }
      pairs[np++] = key_of(a, b);
    }
  }
  long long nbg = llround(p->background_frac * (double)(t / 2));
  for (long long q = 0; q < nbg; ++q) {
    int32_t a = (int32_t)(draw(seed, TAG_GRAPH, 4, 0, 2 * (uint64_t)q) % (uint64_t)n);
    int32_t b = (int32_t)(draw(seed, TAG_GRAPH, 4, 0, 2 * (uint64_t)q + 1) % (uint64_t)n);
    if (a == b) continue;
    if (np == cap_pairs) {
      cap_pairs *= 2;
      uint64_t *grown = (uint64_t *)realloc(pairs, sizeof(uint64_t) * cap_pairs);
      if (!grown) goto out;
      pairs = grown;
    }
    pairs[np++] = key_of(a, b);
  }
  rc = csr_from_pairs(n, pairs, np, row_ptr_out, col_out);
out:
  free(size);
  free(moff);
  free(slot);
  free(coff);
  free(member);
  free(fill);
  free(pairs);
  return rc;
}

/* ---- open-addressing set of pair keys (all-ones = empty) ---------------- */
typedef struct {
  uint64_t *slot;
  uint64_t mask;
} keyset;

static int keyset_init(keyset *s, int64_t want) {
  uint64_t cap = 16;
  while (cap < 4 * (uint64_t)want + 16) cap <<= 1;
  s->slot = (uint64_t *)malloc(sizeof(uint64_t) * cap);
  if (!s->slot) return -1;
  memset(s->slot, 0xff, sizeof(uint64_t) * cap);
  s->mask = cap - 1;
  return 0;
}

static uint64_t mix(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return k;
}

static int keyset_has(const keyset *s, uint64_t k) {
  for (uint64_t h = mix(k) & s->mask;; h = (h + 1) & s->mask) {
    if (s->slot[h] == k) return 1;
    if (s->slot[h] == ~0ull) return 0;
  }
}

/* 1 if inserted, 0 if present */
static int keyset_add(keyset *s, uint64_t k) {
  for (uint64_t h = mix(k) & s->mask;; h = (h + 1) & s->mask) {
    if (s->slot[h] == k) return 0;
    if (s->slot[h] == ~0ull) {
      s->slot[h] = k;
      return 1;
    }
  }
}

static int has_edge_csr(const int64_t *row_ptr, const int32_t *col, int32_t a, int32_t b) {
  int64_t lo = row_ptr[a], hi = row_ptr[a + 1];
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (col[mid] < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < row_ptr[a + 1] && col[lo] == b;
}

int64_t oracle_held_out_pairs(int64_t num_edges, double ratio) {
  return ((int64_t)(ratio * (double)num_edges)) / 2;
}

int oracle_make_held_out(int64_t n, const int64_t *row_ptr, const int32_t *col,
                         double ratio, uint32_t seed, int32_t *ha, int32_t *hb,
                         uint8_t *hy, int32_t *ta, int32_t *tb, uint8_t *ty) {
  if (!row_ptr || !col || ratio < 0 || ratio >= 1 || n < 2) return -1;
  const int64_t E = row_ptr[n] / 2;
  const int64_t p = oracle_held_out_pairs(E, ratio);
  if (E < 2 * p) return -1;
  if ((double)(2 * p) > (double)n * (double)(n - 1) / 2.0 - (double)E) return -1;
  uint64_t *und = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(E + 1));
  keyset held = {0, 0}, test = {0, 0};
  int rc = -1;
  if (!und || keyset_init(&held, 2 * p) || keyset_init(&test, 2 * p)) goto out;
  {
    int64_t q = 0;
    for (int64_t v = 0; v < n; ++v)
      for (int64_t e = row_ptr[v]; e < row_ptr[v + 1]; ++e)
        if (col[e] > v) und[q++] = key_of((int32_t)v, col[e]);
  }
  const uint64_t cap = 1000 * (uint64_t)p + 100000;
  int64_t nh = 0, nt = 0;
  uint64_t t = 0;
  for (int64_t c = 0; c < p; ++t) { /* held-out links */
    if (t > cap) goto out;
    uint64_t k = und[draw(seed, TAG_HELD_OUT, 0, 0, t) % (uint64_t)E];
    if (keyset_add(&held, k)) {
      ha[nh] = (int32_t)(k >> 32), hb[nh] = (int32_t)(uint32_t)k, hy[nh++] = 1;
      ++c;
    }
  }
  t = 0;
  for (int64_t c = 0; c < p; ++t) { /* held-out non-links */
    if (t > cap) goto out;
    int32_t a = (int32_t)(draw(seed, TAG_HELD_OUT, 1, 0, 2 * t) % (uint64_t)n);
    int32_t b = (int32_t)(draw(seed, TAG_HELD_OUT, 1, 0, 2 * t + 1) % (uint64_t)n);
    if (a == b || has_edge_csr(row_ptr, col, a, b)) continue;
    uint64_t k = key_of(a, b);
    if (keyset_add(&held, k)) {
      ha[nh] = (int32_t)(k >> 32), hb[nh] = (int32_t)(uint32_t)k, hy[nh++] = 0;
      ++c;
    }
  }
  t = 0;
  for (int64_t c = 0; c < p; ++t) { /* test links */
    if (t > cap) goto out;
    uint64_t k = und[draw(seed, TAG_HELD_OUT, 2, 0, t) % (uint64_t)E];
    if (keyset_has(&held, k)) continue;
    if (keyset_add(&test, k)) {
      ta[nt] = (int32_t)(k >> 32), tb[nt] = (int32_t)(uint32_t)k, ty[nt++] = 1;
      ++c;
    }
  }
  t = 0;
  for (int64_t c = 0; c < p; ++t) { /* test non-links */
    if (t > cap) goto out;
    int32_t a = (int32_t)(draw(seed, TAG_HELD_OUT, 3, 0, 2 * t) % (uint64_t)n);
    int32_t b = (int32_t)(draw(seed, TAG_HELD_OUT, 3, 0, 2 * t + 1) % (uint64_t)n);
    if (a == b || has_edge_csr(row_ptr, col, a, b)) continue;
    uint64_t k = key_of(a, b);
    if (keyset_has(&held, k)) continue;
    if (keyset_add(&test, k)) {
      ta[nt] = (int32_t)(k >> 32), tb[nt] = (int32_t)(uint32_t)k, ty[nt++] = 0;
      ++c;
    }
  }
  rc = 0;
out:
  free(und);
  free(held.slot);
  free(test.slot);
  return rc;
}

/* phi ~ Gamma(1, 1) as -log(U) (exponential(1) is Gamma(1, 1)), U the
 * 24-bit uniforms of the Philox stream (tag 7, entity = row), and
 * pi = phi / sum(phi) per row (np.h:39-56), rows spread over threads. */
void oracle_init_state_threads(int64_t n, int32_t K, uint32_t seed, float *phi,
                               float *pi, int threads) {
#pragma omp parallel for schedule(static, 256) num_threads(threads > 0 ? threads : 1)
  for (int64_t i = 0; i < n; ++i) {
    float *ph = phi + i * (int64_t)K;
    for (int32_t k = 0; k < K; k += 4) {
      uint32_t ctr[4] = {(uint32_t)(k >> 2), (uint32_t)i, (uint32_t)(i >> 32), 7u};
      uint32_t key[2] = {seed, 0u};
      uint32_t o[4];
      oracle_philox4x32_10(ctr, key, o);
      for (int q = 0; q < 4 && k + q < K; ++q)
        ph[k + q] = -logf(((float)(o[q] >> 8) + 0.5f) * 5.9604644775390625e-08f);
    }
    oracle_normalize_f32(K, ph, pi + i * (int64_t)K);
  }
}

void oracle_free(void *p) { free(p); }
