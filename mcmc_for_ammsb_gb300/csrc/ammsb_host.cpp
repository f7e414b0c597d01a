// ammsb_host.cpp -- host-side data preparation for the GB300 sampler:
// synthetic planted-community graphs, CSR construction, relativity/SNAP text
// I/O and the held-out / test split.  No GPU use; exported through the C ABI
// in include/ammsb_gpu.h.
//
// The reference reads graphs from text (preprocess/relativity.cc:20-200)
// into per-vertex sparse hash sets (data.h:135-313) and carves out the
// held-out and test sets with its sequential RNG (network.cc:503-614).  Here
// the graph is a symmetric CSR with sorted rows -- the layout the GPU binary
// searches -- and every random choice comes from the Philox streams of
// ammsb_rng.h so the result does not depend on hash-table iteration order.
#include <errno.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <unordered_set>
#include <vector>

#include "../../include/ammsb_gpu.h"
#include "ammsb_rng.h"

struct ammsb_graph_buf {
  int64_t n = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col;
};

struct ammsb_split_buf {
  std::vector<int32_t> ha, hb, ta, tb;
  std::vector<uint8_t> hy, ty;
};

namespace {

using ammsb::Stream;

inline double u01_open(uint64_t x) {  // (0, 1)
  return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// LSD radix sort of 64-bit keys whose significant bits are < `bits`.
void radix_sort_u64(std::vector<uint64_t>& keys, int bits) {
  const int kDigit = 11;
  const size_t kBuckets = size_t(1) << kDigit;
  std::vector<uint64_t> tmp(keys.size());
  std::vector<size_t> count(kBuckets);
  for (int shift = 0; shift < bits; shift += kDigit) {
    std::fill(count.begin(), count.end(), 0);
    for (uint64_t k : keys) count[(k >> shift) & (kBuckets - 1)]++;
    size_t sum = 0;
    for (size_t b = 0; b < kBuckets; ++b) {
      size_t c = count[b];
      count[b] = sum;
      sum += c;
    }
    for (uint64_t k : keys) tmp[count[(k >> shift) & (kBuckets - 1)]++] = k;
    keys.swap(tmp);
  }
}

int bits_for(uint64_t v) {
  int b = 1;
  while (b < 64 && (v >> b) != 0) ++b;
  return b;
}

// Symmetric CSR from undirected pairs (self-loops dropped, duplicates merged).
int build_csr(int64_t n, const std::vector<uint64_t>& pairs,
              ammsb_graph_buf* g) {
  // both directions, key = row << 32 | col; sorting gives sorted rows
  std::vector<uint64_t> dir;
  dir.reserve(pairs.size() * 2);
  for (uint64_t p : pairs) {
    uint32_t a = (uint32_t)(p >> 32), b = (uint32_t)p;
    if (a == b) continue;
    if ((int64_t)a >= n || (int64_t)b >= n) return AMMSB_E_ARG;
    dir.push_back(((uint64_t)a << 32) | b);
    dir.push_back(((uint64_t)b << 32) | a);
  }
  radix_sort_u64(dir, 32 + bits_for((uint64_t)(n > 0 ? n - 1 : 0)));
  dir.erase(std::unique(dir.begin(), dir.end()), dir.end());
  g->n = n;
  g->row_ptr.assign((size_t)n + 1, 0);
  g->col.resize(dir.size());
  for (size_t i = 0; i < dir.size(); ++i) {
    g->row_ptr[(dir[i] >> 32) + 1]++;
    g->col[i] = (int32_t)(uint32_t)dir[i];
  }
  for (int64_t v = 0; v < n; ++v) g->row_ptr[v + 1] += g->row_ptr[v];
  return AMMSB_OK;
}

bool has_edge(const ammsb_graph_buf* g, int32_t a, int32_t b) {
  const int32_t* lo = g->col.data() + g->row_ptr[a];
  const int32_t* hi = g->col.data() + g->row_ptr[a + 1];
  const int32_t* p = std::lower_bound(lo, hi, b);
  return p != hi && *p == b;
}

inline uint64_t pair_key(int32_t a, int32_t b) {
  uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
  return ((uint64_t)lo << 32) | hi;
}

}  // namespace

extern "C" {

int ammsb_generate_graph(const ammsb_gen_params* p, ammsb_graph_buf** out) {
  if (!p || !out || p->n < 2 || p->k_true < 1 || p->size_min < 1 ||
      p->size_max < p->size_min || p->zipf_s <= 1.0 || p->p1 < 0 ||
      p->p2 < 0 || p->p1 + p->p2 > 1.0 || p->intra_degree < 0 ||
      p->background_frac < 0 || p->n > INT32_MAX)
    return AMMSB_E_ARG;
  Stream st{p->seed, 0};
  const uint32_t T = ammsb::kTagGraph;
  const int64_t n = p->n, kc = p->k_true;

  // 1. community sizes ~ Zipf(s): continuous Pareto tail, floored, clipped
  std::vector<double> size(kc);
  double size_sum = 0;
  for (int64_t c = 0; c < kc; ++c) {
    double u = u01_open(st.draw_u64(T, 0, 0, (uint64_t)c));
    double s = std::floor((double)p->size_min * std::pow(u, -1.0 / (p->zipf_s - 1.0)));
    s = std::min(std::max(s, (double)p->size_min), (double)p->size_max);
    size[c] = s;
    size_sum += s;
  }
  // 2. memberships per node: 1 / 2 / 3 with p1 / p2 / rest
  std::vector<int64_t> moff(n + 1, 0);
  for (int64_t v = 0; v < n; ++v) {
    double u = u01_open(st.draw_u64(T, 1, 0, (uint64_t)v));
    moff[v + 1] = moff[v] + (u < p->p1 ? 1 : (u < p->p1 + p->p2 ? 2 : 3));
  }
  const int64_t M = moff[n];
  // 3. rescale sizes so the membership slots cover every node's memberships
  std::vector<int32_t> slot;
  slot.reserve(M + kc);
  for (int64_t c = 0; c < kc; ++c) {
    int64_t s = std::max<int64_t>(1, (int64_t)std::llround(size[c] * (double)M / size_sum));
    for (int64_t i = 0; i < s; ++i) slot.push_back((int32_t)c);
  }
  for (uint64_t t = 0; (int64_t)slot.size() < M; ++t)
    slot.push_back((int32_t)(st.draw_u64(T, 2, 1, t) % (uint64_t)kc));
  // Fisher-Yates shuffle, then deal slots to nodes
  for (int64_t i = (int64_t)slot.size() - 1; i > 0; --i) {
    int64_t j = (int64_t)(st.draw_u64(T, 2, 0, (uint64_t)i) % (uint64_t)(i + 1));
    std::swap(slot[i], slot[j]);
  }
  slot.resize(M);
  // 4. member lists per community
  std::vector<int64_t> coff(kc + 1, 0);
  for (int64_t v = 0; v < n; ++v)
    for (int64_t m = moff[v]; m < moff[v + 1]; ++m) coff[slot[m] + 1]++;
  for (int64_t c = 0; c < kc; ++c) coff[c + 1] += coff[c];
  std::vector<int32_t> member(coff[kc]);
  {
    std::vector<int64_t> fill(coff.begin(), coff.end() - 1);
    for (int64_t v = 0; v < n; ++v)
      for (int64_t m = moff[v]; m < moff[v + 1]; ++m)
        member[fill[slot[m]]++] = (int32_t)v;
  }
  // 5. intra-community pairs: round(d * s / 2) uniform member pairs
  std::vector<uint64_t> pairs;
  uint64_t t = 0;
  for (int64_t c = 0; c < kc; ++c) {
    int64_t s = coff[c + 1] - coff[c];
    if (s < 2) continue;
    int64_t np = (int64_t)std::llround(p->intra_degree * (double)s / 2.0);
    for (int64_t q = 0; q < np; ++q, t += 2) {
      int32_t a = member[coff[c] + (int64_t)(st.draw_u64(T, 3, 0, t) % (uint64_t)s)];
      int32_t b = member[coff[c] + (int64_t)(st.draw_u64(T, 3, 0, t + 1) % (uint64_t)s)];
      if (a != b) pairs.push_back(pair_key(a, b));
    }
  }
  // 6. background pairs
  int64_t nbg = (int64_t)std::llround(p->background_frac * (double)(t / 2));
  for (int64_t q = 0; q < nbg; ++q) {
    int32_t a = (int32_t)(st.draw_u64(T, 4, 0, 2 * (uint64_t)q) % (uint64_t)n);
    int32_t b = (int32_t)(st.draw_u64(T, 4, 0, 2 * (uint64_t)q + 1) % (uint64_t)n);
    if (a != b) pairs.push_back(pair_key(a, b));
  }
  auto* g = new ammsb_graph_buf();
  int rc = build_csr(n, pairs, g);
  if (rc != AMMSB_OK) {
    delete g;
    return rc;
  }
  *out = g;
  return AMMSB_OK;
}

int ammsb_graph_from_edges(int64_t n, int64_t n_edges, const int32_t* a,
                           const int32_t* b, ammsb_graph_buf** out) {
  if (!out || n < 1 || n > INT32_MAX || n_edges < 0 || (n_edges > 0 && (!a || !b)))
    return AMMSB_E_ARG;
  std::vector<uint64_t> pairs((size_t)n_edges);
  for (int64_t i = 0; i < n_edges; ++i) {
    if (a[i] < 0 || b[i] < 0 || a[i] >= n || b[i] >= n) return AMMSB_E_ARG;
    pairs[i] = pair_key(a[i], b[i]);
  }
  auto* g = new ammsb_graph_buf();
  int rc = build_csr(n, pairs, g);
  if (rc != AMMSB_OK) {
    delete g;
    return rc;
  }
  *out = g;
  return AMMSB_OK;
}

int ammsb_read_relativity(const char* path, int contiguous,
                          ammsb_graph_buf** out) {
  if (!path || !out) return AMMSB_E_ARG;
  std::ifstream in(path);
  if (!in) return AMMSB_E_ARG;
  std::string line;
  for (int i = 0; i < 4; ++i) std::getline(in, line);  // header, relativity.cc:52-56
  std::vector<int64_t> ea, eb;
  while (std::getline(in, line)) {
    if (line.empty()) continue;
    std::istringstream iss(line);
    int64_t x, y;
    if (!(iss >> x >> y)) return AMMSB_E_ARG;
    ea.push_back(x);
    eb.push_back(y);
  }
  int64_t n = 0;
  std::vector<uint64_t> pairs(ea.size());
  if (contiguous) {
    int64_t mx = -1;
    for (size_t i = 0; i < ea.size(); ++i) {
      if (ea[i] < 0 || eb[i] < 0 || ea[i] > INT32_MAX || eb[i] > INT32_MAX) return AMMSB_E_ARG;
      mx = std::max(mx, std::max(ea[i], eb[i]));
      pairs[i] = pair_key((int32_t)ea[i], (int32_t)eb[i]);
    }
    n = mx + 1;
  } else {
    std::vector<int64_t> ids(ea);
    ids.insert(ids.end(), eb.begin(), eb.end());
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    if ((int64_t)ids.size() > INT32_MAX) return AMMSB_E_ARG;
    n = (int64_t)ids.size();
    for (size_t i = 0; i < ea.size(); ++i) {
      int32_t x = (int32_t)(std::lower_bound(ids.begin(), ids.end(), ea[i]) - ids.begin());
      int32_t y = (int32_t)(std::lower_bound(ids.begin(), ids.end(), eb[i]) - ids.begin());
      pairs[i] = pair_key(x, y);
    }
  }
  if (n < 1) return AMMSB_E_ARG;
  auto* g = new ammsb_graph_buf();
  int rc = build_csr(n, pairs, g);
  if (rc != AMMSB_OK) {
    delete g;
    return rc;
  }
  *out = g;
  return AMMSB_OK;
}

int ammsb_write_relativity(const ammsb_graph_buf* g, const char* path) {
  if (!g || !path) return AMMSB_E_ARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return AMMSB_E_ARG;
  int64_t E = (int64_t)g->col.size() / 2;
  std::fprintf(f, "# Undirected graph: synthetic planted communities\n");
  std::fprintf(f, "# written by libammsb_gpu\n");
  std::fprintf(f, "# Nodes: %lld Edges: %lld\n", (long long)g->n, (long long)E);
  std::fprintf(f, "# FromNodeId\tToNodeId\n");
  for (int64_t v = 0; v < g->n; ++v)
    for (int64_t q = g->row_ptr[v]; q < g->row_ptr[v + 1]; ++q)
      if (g->col[q] > v) std::fprintf(f, "%lld\t%d\n", (long long)v, g->col[q]);
  return std::fclose(f) == 0 ? AMMSB_OK : AMMSB_E_ARG;
}

void ammsb_graph_view(const ammsb_graph_buf* g, ammsb_graph* view) {
  view->n = g->n;
  view->row_ptr = g->row_ptr.data();
  view->col = g->col.data();
}

void ammsb_graph_free(ammsb_graph_buf* g) { delete g; }

// network.cc:503-614.  held_out_size = ratio * E (truncated, network.cc:72);
// p = held_out_size / 2 links and p non-links per set; the test set avoids
// held-out pairs.  Links are drawn uniformly over undirected edges (the
// reference draws one of the 2E directed entries, network.cc:461-489, which
// is the same distribution).
int ammsb_make_held_out(const ammsb_graph_buf* g, double ratio, uint32_t seed,
                        ammsb_split_buf** out) {
  if (!g || !out || ratio < 0 || ratio >= 1) return AMMSB_E_ARG;
  const int64_t n = g->n;
  std::vector<uint64_t> und;  // undirected edges, a < b, ascending
  und.reserve(g->col.size() / 2);
  for (int64_t v = 0; v < n; ++v)
    for (int64_t q = g->row_ptr[v]; q < g->row_ptr[v + 1]; ++q)
      if (g->col[q] > v) und.push_back(pair_key((int32_t)v, g->col[q]));
  const int64_t E = (int64_t)und.size();
  const int64_t held_out_size = (int64_t)(ratio * (double)E);
  const int64_t p = held_out_size / 2;
  if (E < 2 * p || n < 2) return AMMSB_E_ARG;  // network.cc:507-511
  const double nonlinks = (double)n * (double)(n - 1) / 2.0 - (double)E;
  if ((double)(2 * p) > nonlinks) return AMMSB_E_ARG;
  Stream st{seed, 0};
  const uint32_t T = ammsb::kTagHeldOut;
  std::unordered_set<uint64_t> held, test;
  held.reserve(4 * p + 16);
  test.reserve(4 * p + 16);
  auto* s = new ammsb_split_buf();
  auto push = [](std::vector<int32_t>& va, std::vector<int32_t>& vb,
                 std::vector<uint8_t>& vy, uint64_t key, uint8_t y) {
    va.push_back((int32_t)(key >> 32));
    vb.push_back((int32_t)(uint32_t)key);
    vy.push_back(y);
  };
  const uint64_t cap = 1000 * (uint64_t)p + 100000;
  uint64_t t = 0;
  for (int64_t c = 0; c < p; ++t) {  // held-out links
    if (t > cap) { delete s; return AMMSB_E_SAMPLING; }
    uint64_t k = und[st.draw_u64(T, 0, 0, t) % (uint64_t)E];
    if (held.insert(k).second) { push(s->ha, s->hb, s->hy, k, 1); ++c; }
  }
  t = 0;
  for (int64_t c = 0; c < p; ++t) {  // held-out non-links, network.cc:677-697
    if (t > cap) { delete s; return AMMSB_E_SAMPLING; }
    int32_t a = (int32_t)(st.draw_u64(T, 1, 0, 2 * t) % (uint64_t)n);
    int32_t b = (int32_t)(st.draw_u64(T, 1, 0, 2 * t + 1) % (uint64_t)n);
    if (a == b || has_edge(g, a, b)) continue;
    uint64_t k = pair_key(a, b);
    if (held.insert(k).second) { push(s->ha, s->hb, s->hy, k, 0); ++c; }
  }
  t = 0;
  for (int64_t c = 0; c < p; ++t) {  // test links, network.cc:561-593
    if (t > cap) { delete s; return AMMSB_E_SAMPLING; }
    uint64_t k = und[st.draw_u64(T, 2, 0, t) % (uint64_t)E];
    if (held.count(k)) continue;
    if (test.insert(k).second) { push(s->ta, s->tb, s->ty, k, 1); ++c; }
  }
  t = 0;
  for (int64_t c = 0; c < p; ++t) {  // test non-links, network.cc:699-719
    if (t > cap) { delete s; return AMMSB_E_SAMPLING; }
    int32_t a = (int32_t)(st.draw_u64(T, 3, 0, 2 * t) % (uint64_t)n);
    int32_t b = (int32_t)(st.draw_u64(T, 3, 0, 2 * t + 1) % (uint64_t)n);
    if (a == b || has_edge(g, a, b)) continue;
    uint64_t k = pair_key(a, b);
    if (held.count(k)) continue;
    if (test.insert(k).second) { push(s->ta, s->tb, s->ty, k, 0); ++c; }
  }
  *out = s;
  return AMMSB_OK;
}

void ammsb_split_view(const ammsb_split_buf* s, ammsb_edge_set* held_out,
                      ammsb_edge_set* test) {
  if (held_out) {
    held_out->count = (int64_t)s->ha.size();
    held_out->a = s->ha.data();
    held_out->b = s->hb.data();
    held_out->y = s->hy.data();
  }
  if (test) {
    test->count = (int64_t)s->ta.size();
    test->a = s->ta.data();
    test->b = s->tb.data();
    test->y = s->ty.data();
  }
}

void ammsb_split_free(ammsb_split_buf* s) { delete s; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Preprocessed networks: the reference saves a loaded network (graph,
// held-out set with its ratio and size, test set, auxiliary degree data)
// into a directory (network.cc:88-145) and reloads it with input class
// "preprocessed" (network.cc:49-65) instead of reading text and drawing the
// sets again.  Here the directory holds four little-endian binary files:
//   graph.bin     "AMMSBG01", n, nnz (= 2E), row_ptr[n + 1] (int64), col[nnz] (int32)
//   held-out.bin  "AMMSBH01", held_out_ratio (double), count, a[], b[] (int32), y[] (u8)
//   test.bin      "AMMSBT01", count, a[], b[], y[]
//   aux.bin       "AMMSBA01", n, E, largest degree
// Every count is an int64.  The loader checks the tags, the sizes (no
// short or overlong file), the CSR (row_ptr from 0 up to nnz, columns in
// range, each row sorted without repeats and symmetric in count) and the
// pairs (vertices in range, a != b).
namespace {

bool put(FILE* f, const void* p, size_t bytes) { return bytes == 0 || std::fwrite(p, 1, bytes, f) == bytes; }
bool get(FILE* f, void* p, size_t bytes) { return bytes == 0 || std::fread(p, 1, bytes, f) == bytes; }

bool at_eof(FILE* f) {
  unsigned char c;
  return std::fread(&c, 1, 1, f) == 0;
}

struct File {
  FILE* f;
  explicit File(const std::string& path, const char* mode) : f(std::fopen(path.c_str(), mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
  bool close() {
    const bool ok = f && std::fclose(f) == 0;
    f = nullptr;
    return ok;
  }
};

bool write_pairs(FILE* f, const ammsb_edge_set* s) {
  const int64_t c = s ? s->count : 0;
  return put(f, &c, 8) && (c == 0 || (put(f, s->a, 4 * (size_t)c) && put(f, s->b, 4 * (size_t)c) &&
                                      put(f, s->y, (size_t)c)));
}

bool read_pairs(FILE* f, int64_t n, std::vector<int32_t>& a, std::vector<int32_t>& b,
                std::vector<uint8_t>& y) {
  int64_t c = 0;
  if (!get(f, &c, 8) || c < 0 || c > (int64_t)1 << 40) return false;
  a.resize((size_t)c);
  b.resize((size_t)c);
  y.resize((size_t)c);
  if (!get(f, a.data(), 4 * (size_t)c) || !get(f, b.data(), 4 * (size_t)c) || !get(f, y.data(), (size_t)c))
    return false;
  for (int64_t q = 0; q < c; ++q)
    if (a[q] < 0 || b[q] < 0 || a[q] >= n || b[q] >= n || a[q] == b[q] || y[q] > 1) return false;
  return true;
}

}  // namespace

extern "C" {

int ammsb_save_preprocessed(const ammsb_graph* g, const ammsb_edge_set* held_out,
                            const ammsb_edge_set* test, double held_out_ratio, const char* dirname) {
  if (!g || !dirname || g->n < 1 || !g->row_ptr || (g->row_ptr[g->n] > 0 && !g->col))
    return AMMSB_E_ARG;
  if (mkdir(dirname, 0777) != 0 && errno != EEXIST) return AMMSB_E_ARG;
  const std::string dir(dirname);
  const int64_t n = g->n, nnz = g->row_ptr[n];
  {
    File f(dir + "/graph.bin", "wb");
    if (!f.f || !put(f.f, "AMMSBG01", 8) || !put(f.f, &n, 8) || !put(f.f, &nnz, 8) ||
        !put(f.f, g->row_ptr, 8 * (size_t)(n + 1)) || !put(f.f, g->col, 4 * (size_t)nnz) || !f.close())
      return AMMSB_E_ARG;
  }
  {
    File f(dir + "/held-out.bin", "wb");
    if (!f.f || !put(f.f, "AMMSBH01", 8) || !put(f.f, &held_out_ratio, 8) ||
        !write_pairs(f.f, held_out) || !f.close())
      return AMMSB_E_ARG;
  }
  {
    File f(dir + "/test.bin", "wb");
    if (!f.f || !put(f.f, "AMMSBT01", 8) || !write_pairs(f.f, test) || !f.close()) return AMMSB_E_ARG;
  }
  int64_t maxdeg = 0;
  for (int64_t v = 0; v < n; ++v) maxdeg = std::max(maxdeg, g->row_ptr[v + 1] - g->row_ptr[v]);
  const int64_t E = nnz / 2;
  File f(dir + "/aux.bin", "wb");
  if (!f.f || !put(f.f, "AMMSBA01", 8) || !put(f.f, &n, 8) || !put(f.f, &E, 8) || !put(f.f, &maxdeg, 8) ||
      !f.close())
    return AMMSB_E_ARG;
  return AMMSB_OK;
}

int ammsb_load_preprocessed(const char* dirname, ammsb_graph_buf** graph_out,
                            ammsb_split_buf** split_out, double* held_out_ratio) {
  if (!dirname || !graph_out || !split_out) return AMMSB_E_ARG;
  const std::string dir(dirname);
  char tag[8];
  auto g = std::make_unique<ammsb_graph_buf>();
  {
    File f(dir + "/graph.bin", "rb");
    int64_t n = 0, nnz = 0;
    if (!f.f || !get(f.f, tag, 8) || std::memcmp(tag, "AMMSBG01", 8) != 0 || !get(f.f, &n, 8) ||
        !get(f.f, &nnz, 8) || n < 1 || n > (int64_t)INT32_MAX || nnz < 0 || nnz % 2 != 0 ||
        nnz > (int64_t)1 << 40)
      return AMMSB_E_ARG;
    g->n = n;
    g->row_ptr.resize((size_t)n + 1);
    g->col.resize((size_t)nnz);
    if (!get(f.f, g->row_ptr.data(), 8 * (size_t)(n + 1)) || !get(f.f, g->col.data(), 4 * (size_t)nnz) ||
        !at_eof(f.f))
      return AMMSB_E_ARG;
    if (g->row_ptr[0] != 0 || g->row_ptr[n] != nnz) return AMMSB_E_ARG;
    for (int64_t v = 0; v < n; ++v) {
      const int64_t lo = g->row_ptr[v], hi = g->row_ptr[v + 1];
      if (hi < lo || hi > nnz) return AMMSB_E_ARG;
      for (int64_t q = lo; q < hi; ++q)
        if (g->col[q] < 0 || g->col[q] >= n || g->col[q] == v || (q > lo && g->col[q] <= g->col[q - 1]))
          return AMMSB_E_ARG;
    }
  }
  auto s = std::make_unique<ammsb_split_buf>();
  double ratio = 0.0;
  {
    File f(dir + "/held-out.bin", "rb");
    if (!f.f || !get(f.f, tag, 8) || std::memcmp(tag, "AMMSBH01", 8) != 0 || !get(f.f, &ratio, 8) ||
        !(ratio >= 0.0 && ratio < 1.0) || !read_pairs(f.f, g->n, s->ha, s->hb, s->hy) || !at_eof(f.f))
      return AMMSB_E_ARG;
  }
  {
    File f(dir + "/test.bin", "rb");
    if (!f.f || !get(f.f, tag, 8) || std::memcmp(tag, "AMMSBT01", 8) != 0 ||
        !read_pairs(f.f, g->n, s->ta, s->tb, s->ty) || !at_eof(f.f))
      return AMMSB_E_ARG;
  }
  {
    File f(dir + "/aux.bin", "rb");
    int64_t n = 0, E = 0, maxdeg = 0;
    if (!f.f || !get(f.f, tag, 8) || std::memcmp(tag, "AMMSBA01", 8) != 0 || !get(f.f, &n, 8) ||
        !get(f.f, &E, 8) || !get(f.f, &maxdeg, 8) || !at_eof(f.f) || n != g->n ||
        E != (int64_t)g->col.size() / 2)
      return AMMSB_E_ARG;
  }
  // a symmetric graph: every entry (v, u) has its (u, v)
  for (int64_t v = 0; v < g->n; ++v)
    for (int64_t q = g->row_ptr[v]; q < g->row_ptr[v + 1]; ++q)
      if (!has_edge(g.get(), g->col[q], (int32_t)v)) return AMMSB_E_ARG;
  if (held_out_ratio) *held_out_ratio = ratio;
  *graph_out = g.release();
  *split_out = s.release();
  return AMMSB_OK;
}

}  // extern "C"
