/*
 * ORACLE — test infrastructure only (see beam_oracle.h). Plain-C restatement
 * of githubofzby/beam's recommended merge loop. Each function names the
 * reference lines it restates; data structures are this file's own
 * (flat per-row arrays, sort-based bucketing, dense per-group pair tables)
 * and only the arithmetic and the decision order follow the reference.
 */
#define _POSIX_C_SOURCE 200809L
#include "beam_oracle.h"

#include <limits.h>
#include <omp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static __thread char g_err[512];

static void set_err(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

const char* beam_oracle_last_error(void) { return g_err; }

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec * 1e3 + (double)ts.tv_nsec * 1e-6;
}

static void* xmalloc(size_t bytes) {
  void* p = malloc(bytes ? bytes : 1);
  if (!p) {
    fprintf(stderr, "oracle: out of memory (%zu bytes)\n", bytes);
    abort();
  }
  return p;
}

static void* xcalloc(size_t count, size_t size) {
  void* p = calloc(count ? count : 1, size ? size : 1);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

/* ------------------------------------------------------------ state */

typedef struct {
  int32_t* nb;
  int64_t* cnt;
  int32_t len, cap;
} qrow;

typedef struct {
  int32_t t, i;
  int64_t e;
} tentry;

typedef struct {
  int32_t other;
  int32_t lo, hi;
  int64_t pg;
  double ratio;
} ranked;

typedef struct {
  int32_t a, b;
  int64_t gain, before;
} cand;

typedef struct {
  int32_t rep, idx;
} repidx;

typedef struct {
  tentry* ent;
  size_t ent_cap;
  int64_t* pmat;
  uint8_t* fmat;
  size_t mat_cap;
  int64_t* old;
  ranked* rk;
  size_t rk_cap;
  repidx* map;
  size_t map_cap;
} workspace;

typedef struct {
  int32_t* q;
  int32_t g;
  cand* c;
  int64_t nc;
  uint64_t examined, view_nnz;
} prepared;

struct beam_oracle {
  int32_t n;
  int64_t arcs;
  const int64_t* row_ptr;
  const int32_t* col;
  beam_oracle_config cfg;
  /* QuotientGraph state (include/quotient_graph.hpp:193-200) */
  int64_t* qsize;
  int64_t* qint;
  uint8_t* qact;
  qrow* rows;
  /* Sweg partition lists (include/sweg.hpp:689-695) */
  int32_t *I, *J, *S, *tail;
  int32_t* sizes_by_rep;
  /* Divide output (include/sweg.hpp:749-752) */
  int32_t* reps;
  int64_t n_active;
  int32_t *gstart, *glen;
  int64_t n_groups;
  int32_t dim_order[256];
  uint64_t* hbuf;
  beam_oracle_stats st;
  int nthreads;
  workspace* ws;
  int err;
};

/* ------------------------------------------------------ arithmetic */

/* CostOracle::BlockCost (src/cost_oracle.cpp:93-110): min(e, 1 + cap - e),
 * cap = s(s-1)/2 for an internal block, s_a * s_b across; capacity overflow,
 * negative inputs or e > cap are errors. */
static inline int64_t block_cost(int64_t sa, int64_t sb, int64_t e, int internal, int* err) {
  if (sa < 0 || sb < 0 || e < 0 || (internal && sa != sb)) {
    *err = 1;
    return 0;
  }
  const __int128 capw = internal ? (__int128)sa * (sa - 1) / 2 : (__int128)sa * sb;
  if (capw > (__int128)INT64_MAX || (__int128)e > capw) {
    *err = 1;
    return 0;
  }
  const int64_t alt = 1 + (int64_t)capw - e;
  return e < alt ? e : alt;
}

/* Sweg::EncodeCostForPair (src/sweg.cpp:1423-1433), plain int64 arithmetic. */
static inline int64_t encode_cost_for_pair(int32_t rep_u, int64_t size_u, int32_t rep_x,
                                           int64_t size_x, int64_t edges) {
  const int64_t cap = rep_u == rep_x ? size_u * (size_u - 1) / 2 : size_u * size_x;
  const int64_t alt = 1 + cap - edges;
  return edges < alt ? edges : alt;
}

/* Sweg::SplitMix64 (src/sweg.cpp:2290-2295). */
static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}

/* Sweg::HashRank64 / DimRank / FallbackRank (src/sweg.cpp:731-752). */
static inline uint64_t hash_rank(uint64_t seed, int32_t node, int32_t dim, int32_t iter) {
  uint64_t x = seed;
  x ^= 0x9e3779b97f4a7c15ULL * (uint64_t)(node + 1);
  x ^= 0xbf58476d1ce4e5b9ULL * (uint64_t)(dim + 1);
  x ^= 0x94d049bb133111ebULL * (uint64_t)(iter + 1);
  return splitmix64(x);
}
static inline uint64_t dim_rank(uint64_t seed, int32_t dim, int32_t iter) {
  uint64_t x = seed;
  x ^= 0x9e3779b97f4a7c15ULL * (uint64_t)(dim + 1);
  x ^= 0xbf58476d1ce4e5b9ULL * (uint64_t)(iter + 1);
  return splitmix64(x);
}
static inline uint64_t fallback_rank(uint64_t seed, int32_t rep, int32_t iter) {
  uint64_t x = seed;
  x ^= 0x9e3779b97f4a7c15ULL * (uint64_t)(rep + 1);
  x ^= 0xbf58476d1ce4e5b9ULL * (uint64_t)(iter + 1);
  x ^= 0xd6e8feb86659fd93ULL;
  return splitmix64(x);
}

/* ------------------------------------------------------- rows */

static void row_reserve(qrow* r, int32_t need) {
  if (need <= r->cap) return;
  int32_t cap = r->cap ? r->cap : 4;
  while (cap < need) cap = cap * 2;
  r->nb = (int32_t*)realloc(r->nb, sizeof(int32_t) * (size_t)cap);
  r->cnt = (int64_t*)realloc(r->cnt, sizeof(int64_t) * (size_t)cap);
  if (!r->nb || !r->cnt) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  r->cap = cap;
}

static inline int32_t row_lower_bound(const qrow* r, int32_t key) {
  int32_t lo = 0, hi = r->len;
  while (lo < hi) {
    const int32_t mid = lo + (hi - lo) / 2;
    if (r->nb[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* QuotientGraph::RowEdgeCount (src/quotient_graph.cpp:185-191). */
static inline int64_t row_count(const qrow* r, int32_t key) {
  const int32_t p = row_lower_bound(r, key);
  return (p < r->len && r->nb[p] == key) ? r->cnt[p] : 0;
}

/* QuotientGraph::SetRowEdgeCount (src/quotient_graph.cpp:193-217): update,
 * erase on zero, or insert at the sorted position. */
static void row_set(qrow* r, int32_t key, int64_t count) {
  const int32_t p = row_lower_bound(r, key);
  if (p < r->len && r->nb[p] == key) {
    if (count == 0) {
      memmove(r->nb + p, r->nb + p + 1, sizeof(int32_t) * (size_t)(r->len - p - 1));
      memmove(r->cnt + p, r->cnt + p + 1, sizeof(int64_t) * (size_t)(r->len - p - 1));
      r->len--;
    } else {
      r->cnt[p] = count;
    }
  } else if (count != 0) {
    row_reserve(r, r->len + 1);
    memmove(r->nb + p + 1, r->nb + p, sizeof(int32_t) * (size_t)(r->len - p));
    memmove(r->cnt + p + 1, r->cnt + p, sizeof(int64_t) * (size_t)(r->len - p));
    r->nb[p] = key;
    r->cnt[p] = count;
    r->len++;
  }
}

/* ------------------------------------------------------ lifecycle */

void beam_oracle_default_config(beam_oracle_config* cfg) {
  cfg->top_k = 16;
  cfg->group_batch_size = 64;
  cfg->divide_hash_dims = 16;
  cfg->divide_max_group = 512;
  cfg->ea_use_threshold = 1;
  cfg->seed = 1;
  cfg->threads = 0;
}

static int cmp_i64(const void* x, const void* y) {
  const int64_t a = *(const int64_t*)x, b = *(const int64_t*)y;
  return a < b ? -1 : (a > b ? 1 : 0);
}

/* QuotientGraph::Initialize + Rebuild with identity labels
 * (src/quotient_graph.cpp:72-145): cross rows hold one count per arc u<v,
 * counts of repeated arcs are summed, rows sorted by neighbour. */
static int quotient_init(beam_oracle* o) {
  const int32_t n = o->n;
  int32_t* deg = (int32_t*)xcalloc((size_t)n, sizeof(int32_t));
  for (int32_t u = 0; u < n; ++u) {
    for (int64_t k = o->row_ptr[u]; k < o->row_ptr[u + 1]; ++k) {
      const int32_t v = o->col[k];
      if (v < 0 || v >= n || v == u) {
        free(deg);
        set_err("QuotientGraph requires a loop-free graph with valid neighbors");
        return -1;
      }
      if (u < v) {
        deg[u]++;
        deg[v]++;
      }
    }
  }
  for (int32_t u = 0; u < n; ++u) {
    o->qsize[u] = 1;
    o->qint[u] = 0;
    o->qact[u] = 1;
    row_reserve(&o->rows[u], deg[u] > 0 ? deg[u] : 1);
    o->rows[u].len = 0;
  }
  for (int32_t u = 0; u < n; ++u) {
    for (int64_t k = o->row_ptr[u]; k < o->row_ptr[u + 1]; ++k) {
      const int32_t v = o->col[k];
      if (u < v) {
        qrow* ru = &o->rows[u];
        qrow* rv = &o->rows[v];
        ru->nb[ru->len] = v;
        ru->cnt[ru->len++] = 1;
        rv->nb[rv->len] = u;
        rv->cnt[rv->len++] = 1;
      }
    }
  }
  /* sort + merge duplicates (rows are mostly sorted already) */
  int64_t* tmp = NULL;
  size_t tmp_cap = 0;
  for (int32_t u = 0; u < n; ++u) {
    qrow* r = &o->rows[u];
    if ((size_t)r->len > tmp_cap) {
      tmp_cap = (size_t)r->len;
      tmp = (int64_t*)realloc(tmp, sizeof(int64_t) * tmp_cap);
    }
    for (int32_t k = 0; k < r->len; ++k) tmp[k] = r->nb[k];
    qsort(tmp, (size_t)r->len, sizeof(int64_t), cmp_i64);
    int32_t out = 0;
    for (int32_t k = 0; k < r->len; ++k) {
      if (out > 0 && r->nb[out - 1] == (int32_t)tmp[k]) {
        r->cnt[out - 1] += 1;
      } else {
        r->nb[out] = (int32_t)tmp[k];
        r->cnt[out] = 1;
        ++out;
      }
    }
    r->len = out;
  }
  free(tmp);
  free(deg);
  return 0;
}

static void ensure_ws(workspace* w, size_t entries, int32_t g) {
  if (entries > w->ent_cap) {
    w->ent_cap = entries * 2;
    free(w->ent);
    w->ent = (tentry*)xmalloc(sizeof(tentry) * w->ent_cap);
  }
  const size_t gg = (size_t)g * (size_t)g;
  if (gg > w->mat_cap) {
    w->mat_cap = gg;
    free(w->pmat);
    free(w->fmat);
    free(w->old);
    free(w->rk);
    free(w->map);
    w->pmat = (int64_t*)xmalloc(sizeof(int64_t) * gg);
    w->fmat = (uint8_t*)xmalloc(gg);
    w->old = (int64_t*)xmalloc(sizeof(int64_t) * (size_t)g);
    w->rk = (ranked*)xmalloc(sizeof(ranked) * (size_t)g);
    w->map = (repidx*)xmalloc(sizeof(repidx) * (size_t)g);
  }
}

beam_oracle* beam_oracle_create(int32_t n, int64_t arcs, const int64_t* row_ptr,
                                const int32_t* col_idx, const beam_oracle_config* cfg) {
  if (n <= 0 || !row_ptr || (arcs > 0 && !col_idx) || row_ptr[n] != arcs) {
    set_err("invalid CSR graph shape");
    return NULL;
  }
  beam_oracle* o = (beam_oracle*)xcalloc(1, sizeof(beam_oracle));
  o->n = n;
  o->arcs = arcs;
  o->row_ptr = row_ptr;
  o->col = col_idx;
  if (cfg) o->cfg = *cfg; else beam_oracle_default_config(&o->cfg);
  if (o->cfg.divide_hash_dims <= 0) o->cfg.divide_hash_dims = 16;
  if (o->cfg.divide_hash_dims > 256) o->cfg.divide_hash_dims = 256;
  if (o->cfg.divide_max_group <= 0) o->cfg.divide_max_group = 512;
  if (o->cfg.group_batch_size < 1) o->cfg.group_batch_size = 1;
  o->qsize = (int64_t*)xcalloc((size_t)n, sizeof(int64_t));
  o->qint = (int64_t*)xcalloc((size_t)n, sizeof(int64_t));
  o->qact = (uint8_t*)xcalloc((size_t)n, 1);
  o->rows = (qrow*)xcalloc((size_t)n, sizeof(qrow));
  o->I = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->J = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->S = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->tail = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->sizes_by_rep = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->reps = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->gstart = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->glen = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  o->hbuf = (uint64_t*)xmalloc(sizeof(uint64_t) * (size_t)n * 2);
  /* Sweg::Sweg (src/sweg.cpp:142-154) */
  for (int32_t i = 0; i < n; ++i) {
    o->I[i] = i;
    o->J[i] = -1;
    o->S[i] = i;
    o->tail[i] = i;
    o->sizes_by_rep[i] = 1;
  }
  o->nthreads = o->cfg.threads > 0 ? o->cfg.threads : omp_get_max_threads();
  if (o->nthreads < 1) o->nthreads = 1;
  o->ws = (workspace*)xcalloc((size_t)o->nthreads, sizeof(workspace));
  if (quotient_init(o) != 0) {
    beam_oracle_free(o);
    return NULL;
  }
  return o;
}

void beam_oracle_free(beam_oracle* o) {
  if (!o) return;
  for (int32_t i = 0; i < o->n; ++i) {
    free(o->rows[i].nb);
    free(o->rows[i].cnt);
  }
  for (int t = 0; t < o->nthreads; ++t) {
    free(o->ws[t].ent);
    free(o->ws[t].pmat);
    free(o->ws[t].fmat);
    free(o->ws[t].old);
    free(o->ws[t].rk);
    free(o->ws[t].map);
  }
  free(o->ws);
  free(o->rows);
  free(o->qsize);
  free(o->qint);
  free(o->qact);
  free(o->I);
  free(o->J);
  free(o->S);
  free(o->tail);
  free(o->sizes_by_rep);
  free(o->reps);
  free(o->gstart);
  free(o->glen);
  free(o->hbuf);
  free(o);
}

/* ------------------------------------------------ exact merge gain */

typedef struct {
  uint64_t raw_a, raw_b, uni, ovl;
} gain_work;

/* QuotientGraph::ExactMergeGainPersistentImpl (src/quotient_graph.cpp:340-462):
 * two-pointer union of rows a and b; a and b themselves record e_ab; every
 * other neighbour x adds BlockCost(s_a,s_x,e_a)+BlockCost(s_b,s_x,e_b) before
 * if shared, the one-sided BlockCost otherwise, and BlockCost(s_w,s_x,e_a+e_b)
 * after; then the three internal/ab before-terms and the merged internal
 * after-term. */
static int exact_gain(const beam_oracle* o, int32_t a, int32_t b, int64_t* gain, int64_t* before_out,
                      gain_work* work) {
  int err = 0;
  if (a < 0 || b < 0 || a >= o->n || b >= o->n || !o->qact[a] || !o->qact[b]) return -1;
  if (a == b) return -2;
  const int64_t sa = o->qsize[a], sb = o->qsize[b];
  const int64_t sw = sa + sb;
  const qrow* ra = &o->rows[a];
  const qrow* rb = &o->rows[b];
  int64_t before = 0, after = 0, eab_a = 0, eab_b = 0;
  uint64_t uni = 0, ovl = 0;
  int32_t ia = 0, ib = 0;
  while (ia < ra->len || ib < rb->len) {
    int32_t x;
    int64_t ea = 0, eb = 0;
    int overlap = 0;
    if (ib >= rb->len || (ia < ra->len && ra->nb[ia] < rb->nb[ib])) {
      x = ra->nb[ia];
      ea = ra->cnt[ia++];
    } else if (ia >= ra->len || rb->nb[ib] < ra->nb[ia]) {
      x = rb->nb[ib];
      eb = rb->cnt[ib++];
    } else {
      x = ra->nb[ia];
      ea = ra->cnt[ia++];
      eb = rb->cnt[ib++];
      overlap = 1;
    }
    if (x == b) {
      eab_a = ea;
      continue;
    }
    if (x == a) {
      eab_b = eb;
      continue;
    }
    const int64_t sx = o->qsize[x];
    if (overlap) {
      before += block_cost(sa, sx, ea, 0, &err) + block_cost(sb, sx, eb, 0, &err);
      ++ovl;
    } else {
      before += ea != 0 ? block_cost(sa, sx, ea + eb, 0, &err) : block_cost(sb, sx, ea + eb, 0, &err);
    }
    after += block_cost(sw, sx, ea + eb, 0, &err);
    ++uni;
  }
  if (eab_a != eab_b) return -3;
  before += block_cost(sa, sa, o->qint[a], 1, &err);
  before += block_cost(sb, sb, o->qint[b], 1, &err);
  before += block_cost(sa, sb, eab_a, 0, &err);
  after += block_cost(sw, sw, o->qint[a] + o->qint[b] + eab_a, 1, &err);
  if (err) return -4;
  if (work) {
    work->raw_a += (uint64_t)ra->len;
    work->raw_b += (uint64_t)rb->len;
    work->uni += uni;
    work->ovl += ovl;
  }
  *gain = before - after;
  *before_out = before;
  return 0;
}

int beam_oracle_exact_gain(const beam_oracle* o, int32_t a, int32_t b, int64_t* gain, int64_t* before) {
  const int rc = exact_gain(o, a, b, gain, before, NULL);
  if (rc == -1) set_err("quotient supernode is inactive or out of range");
  if (rc == -2) set_err("merge endpoints must differ");
  if (rc == -3) set_err("asymmetric quotient edge count during scoring");
  if (rc == -4) set_err("merge gain cost overflow");
  return rc;
}

/* ------------------------------------------------ quotient merge */

/* QuotientGraph::Merge (src/quotient_graph.cpp:628-742): sizes and internal
 * counts added, keep<->remove entries dropped, keep's row becomes the
 * count-summed union of both rows, every neighbour row of remove trades its
 * remove entry for keep (count = merged count); returns 2 + 3|row(remove)|. */
static uint64_t quotient_merge(beam_oracle* o, int32_t keep, int32_t remove) {
  qrow* rk = &o->rows[keep];
  qrow* rr = &o->rows[remove];
  const int64_t cross = row_count(rk, remove);
  o->qsize[keep] += o->qsize[remove];
  o->qint[keep] += o->qint[remove] + cross;
  row_set(rk, remove, 0);
  row_set(rr, keep, 0);
  const int32_t lk = rk->len, lr = rr->len;
  int32_t* nb = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)(lk + lr + 1));
  int64_t* ct = (int64_t*)xmalloc(sizeof(int64_t) * (size_t)(lk + lr + 1));
  int32_t i = 0, j = 0, out = 0;
  while (i < lk || j < lr) {
    if (j >= lr || (i < lk && rk->nb[i] < rr->nb[j])) {
      nb[out] = rk->nb[i];
      ct[out++] = rk->cnt[i++];
    } else if (i >= lk || rr->nb[j] < rk->nb[i]) {
      nb[out] = rr->nb[j];
      ct[out++] = rr->cnt[j++];
    } else {
      nb[out] = rk->nb[i];
      ct[out++] = rk->cnt[i++] + rr->cnt[j++];
    }
  }
  free(rk->nb);
  free(rk->cnt);
  rk->nb = nb;
  rk->cnt = ct;
  rk->len = out;
  rk->cap = lk + lr + 1;
  uint64_t touched = 2;
  for (int32_t k = 0; k < lr; ++k) {
    const int32_t x = rr->nb[k];
    const int64_t merged = row_count(rk, x);
    row_set(&o->rows[x], remove, 0);
    row_set(&o->rows[x], keep, merged);
    touched += 3;
  }
  rr->len = 0;
  o->qsize[remove] = 0;
  o->qint[remove] = 0;
  o->qact[remove] = 0;
  return touched;
}

/* Sweg::Update_S (src/sweg.cpp:2977-3015): quotient merge, then B's member
 * list is appended after A's and every member is relabelled to A's head. */
static void update_s(beam_oracle* o, int32_t A, int32_t B) {
  if (o->I[A] == -1 || o->I[B] == -1) return;
  o->st.update_touched_quotient_entries += quotient_merge(o, A, B);
  o->J[o->tail[A]] = o->I[B];
  o->tail[A] = o->tail[B];
  o->I[B] = -1;
  const int32_t head = o->I[A];
  int32_t count = 0;
  for (int32_t node = head; node != -1; node = o->J[node]) {
    o->S[node] = head;
    ++count;
  }
  o->sizes_by_rep[A] = count;
  o->sizes_by_rep[B] = 0;
}

int beam_oracle_merge_pair(beam_oracle* o, int32_t keep, int32_t remove) {
  if (keep < 0 || remove < 0 || keep >= o->n || remove >= o->n || keep == remove ||
      !o->qact[keep] || !o->qact[remove]) {
    set_err("invalid merge endpoints");
    return -1;
  }
  update_s(o, keep, remove);
  return 0;
}

/* --------------------------------------------------------- divide */

typedef struct {
  uint64_t h;
  int32_t rep;
} hrep;

static int cmp_hrep(const void* x, const void* y) {
  const hrep* a = (const hrep*)x;
  const hrep* b = (const hrep*)y;
  if (a->h != b->h) return a->h < b->h ? -1 : 1;
  return a->rep < b->rep ? -1 : (a->rep > b->rep ? 1 : 0);
}

static void push_group(beam_oracle* o, int32_t start, int32_t len) {
  o->gstart[o->n_groups] = start;
  o->glen[o->n_groups] = len;
  o->n_groups++;
  if (len > o->st.divide_max_group_size) o->st.divide_max_group_size = len;
}

/* Sweg::SupernodeMinHash via NodeShingleDim (src/sweg.cpp:754-784): minimum
 * over member nodes v and their CSR neighbours u of HashRank64(., dim, iter). */
static uint64_t supernode_minhash(const beam_oracle* o, int32_t rep, int32_t dim, int32_t iter) {
  uint64_t best = UINT64_MAX;
  for (int32_t v = o->I[rep]; v != -1; v = o->J[v]) {
    uint64_t s = hash_rank(o->cfg.seed, v, dim, iter);
    for (int64_t k = o->row_ptr[v]; k < o->row_ptr[v + 1]; ++k) {
      const uint64_t h = hash_rank(o->cfg.seed, o->col[k], dim, iter);
      if (h < s) s = h;
    }
    if (s < best) best = s;
  }
  return best;
}

/* Sweg::FallbackSplitGroup (src/sweg.cpp:786-810). */
static void fallback_split(beam_oracle* o, int32_t l, int32_t r, int32_t iter) {
  if (l >= r) return;
  o->st.divide_fallback_splits++;
  hrep* tmp = (hrep*)xmalloc(sizeof(hrep) * (size_t)(r - l));
  for (int32_t k = l; k < r; ++k) {
    tmp[k - l].h = fallback_rank(o->cfg.seed, o->reps[k], iter);
    tmp[k - l].rep = o->reps[k];
  }
  qsort(tmp, (size_t)(r - l), sizeof(hrep), cmp_hrep);
  for (int32_t k = l; k < r; ++k) o->reps[k] = tmp[k - l].rep;
  free(tmp);
  for (int32_t s = l; s < r; s += o->cfg.divide_max_group) {
    const int32_t e = s + o->cfg.divide_max_group < r ? s + o->cfg.divide_max_group : r;
    if (e > s) push_group(o, s, e - s);
  }
}

/* Sweg::SplitGroupByHashDims (src/sweg.cpp:812-851): sort the range by
 * (min-hash of dimension dim_order[depth], rep), recurse on equal-hash runs
 * until a run has at most divide_max_group reps. */
static void split_group(beam_oracle* o, int32_t l, int32_t r, int32_t depth, int32_t iter) {
  if (l >= r) return;
  const int32_t size = r - l;
  if (size <= o->cfg.divide_max_group) {
    push_group(o, l, size);
    return;
  }
  if (depth >= o->cfg.divide_hash_dims) {
    fallback_split(o, l, r, iter);
    return;
  }
  const int32_t dim = o->dim_order[depth];
  hrep* tmp = (hrep*)xmalloc(sizeof(hrep) * (size_t)size);
#pragma omp parallel for schedule(dynamic, 256) if (size > 4096) num_threads(o->nthreads)
  for (int32_t k = l; k < r; ++k) {
    tmp[k - l].h = supernode_minhash(o, o->reps[k], dim, iter);
    tmp[k - l].rep = o->reps[k];
  }
  qsort(tmp, (size_t)size, sizeof(hrep), cmp_hrep);
  for (int32_t k = l; k < r; ++k) o->reps[k] = tmp[k - l].rep;
  int32_t begin = 0;
  while (begin < size) {
    int32_t end = begin + 1;
    while (end < size && tmp[end].h == tmp[begin].h) ++end;
    /* free the scratch before recursing deeper */
    split_group(o, l + begin, l + end, depth + 1, iter);
    begin = end;
  }
  free(tmp);
}

typedef struct {
  uint64_t r;
  int32_t d;
} dimr;

static int cmp_dimr(const void* x, const void* y) {
  const dimr* a = (const dimr*)x;
  const dimr* b = (const dimr*)y;
  if (a->r != b->r) return a->r < b->r ? -1 : 1;
  return a->d < b->d ? -1 : (a->d > b->d ? 1 : 0);
}

/* Sweg::Divide (src/sweg.cpp:853-890). */
int beam_oracle_divide(beam_oracle* o, int iter) {
  o->n_active = 0;
  o->n_groups = 0;
  for (int32_t rep = 0; rep < o->n; ++rep) {
    if (o->I[rep] != -1) o->reps[o->n_active++] = rep;
  }
  dimr dr[256];
  for (int32_t d = 0; d < o->cfg.divide_hash_dims; ++d) {
    dr[d].r = dim_rank(o->cfg.seed, d, iter);
    dr[d].d = d;
  }
  qsort(dr, (size_t)o->cfg.divide_hash_dims, sizeof(dimr), cmp_dimr);
  for (int32_t d = 0; d < o->cfg.divide_hash_dims; ++d) o->dim_order[d] = dr[d].d;
  split_group(o, 0, (int32_t)o->n_active, 0, iter);
  o->st.groups_last = (uint64_t)o->n_groups;
  o->st.active_supernodes_last = (uint64_t)o->n_active;
  return 0;
}

int64_t beam_oracle_group_count(const beam_oracle* o) { return o->n_groups; }
int64_t beam_oracle_active_count(const beam_oracle* o) { return o->n_active; }

int beam_oracle_groups(const beam_oracle* o, int32_t* order, int32_t* starts, int32_t* lengths) {
  if (order) memcpy(order, o->reps, sizeof(int32_t) * (size_t)o->n_active);
  if (starts) memcpy(starts, o->gstart, sizeof(int32_t) * (size_t)o->n_groups);
  if (lengths) memcpy(lengths, o->glen, sizeof(int32_t) * (size_t)o->n_groups);
  return 0;
}

/* ------------------------------------------------------- prepare */

static int cmp_tentry(const void* x, const void* y) {
  const tentry* a = (const tentry*)x;
  const tentry* b = (const tentry*)y;
  if (a->t != b->t) return a->t < b->t ? -1 : 1;
  return a->i < b->i ? -1 : (a->i > b->i ? 1 : 0);
}

/* ranked_better (src/sweg.cpp:1926-1938): ratio desc, proxy gain desc,
 * rep_lo asc, rep_hi asc. */
static int cmp_ranked(const void* x, const void* y) {
  const ranked* a = (const ranked*)x;
  const ranked* b = (const ranked*)y;
  if (a->ratio != b->ratio) return a->ratio > b->ratio ? -1 : 1;
  if (a->pg != b->pg) return a->pg > b->pg ? -1 : 1;
  if (a->lo != b->lo) return a->lo < b->lo ? -1 : 1;
  if (a->hi != b->hi) return a->hi < b->hi ? -1 : 1;
  return 0;
}

static int cmp_repidx(const void* x, const void* y) {
  const repidx* a = (const repidx*)x;
  const repidx* b = (const repidx*)y;
  return a->rep < b->rep ? -1 : (a->rep > b->rep ? 1 : 0);
}

static int32_t find_idx(const repidx* map, int32_t g, int32_t rep) {
  int32_t lo = 0, hi = g;
  while (lo < hi) {
    const int32_t mid = lo + (hi - lo) / 2;
    if (map[mid].rep < rep) lo = mid + 1; else hi = mid;
  }
  return (lo < g && map[lo].rep == rep) ? map[lo].idx : -1;
}

/* PrepareBatchEncodingAwareGroupWithWorkspace, persistent state with the
 * legacy EA-proxy (src/sweg.cpp:1598-1727, 1800-1999). Member row views carry
 * the virtual internal entry (rep, 2*internal) (src/quotient_graph.cpp:596-616).
 *  - approx_old[i] = sum of EncodeCostForPair over i's view entries
 *  - for every target t and every two members a<b whose views hold t
 *    (t not a's or b's own rep): proxy[a,b] += max(0, old - new) with
 *    old = ECP(a,t)+ECP(b,t), new = ECP(a with s_a+s_b, e_a+e_b)
 *  - proxy[i,j] += e(i,j) for in-group neighbours
 *  - each member keeps its top_k partners by ratio = proxy/max(1,old_a+old_b)
 *  - the union of kept pairs, sorted by (a_idx, b_idx). */
static int prepare_group(const beam_oracle* o, workspace* w, const int32_t* q, int32_t g,
                         prepared* out) {
  out->q = (int32_t*)q;
  out->g = g;
  out->c = NULL;
  out->nc = 0;
  out->examined = 0;
  out->view_nnz = 0;
  if (g < 2) return 0;
  int32_t top_k = o->cfg.top_k < g - 1 ? o->cfg.top_k : g - 1; /* max(1, min(top_k, g-1)) */
  if (top_k < 1) top_k = 1;
  size_t entries = 0;
  for (int32_t i = 0; i < g; ++i) entries += (size_t)o->rows[q[i]].len + 1;
  ensure_ws(w, entries, g);
  /* approximate old costs and target entries */
  size_t ne = 0;
  for (int32_t i = 0; i < g; ++i) {
    const int32_t rep = q[i];
    const int64_t si = o->qsize[rep];
    const qrow* r = &o->rows[rep];
    const int64_t internal = o->qint[rep];
    const int32_t ipos = row_lower_bound(r, rep);
    int64_t old = 0;
    for (int32_t k = 0; k <= r->len; ++k) {
      int32_t t;
      int64_t e;
      if (k == ipos && internal > 0) {
        t = rep;
        e = 2 * internal;
        old += encode_cost_for_pair(rep, si, t, (int64_t)o->sizes_by_rep[t], e);
        w->ent[ne].t = t;
        w->ent[ne].i = i;
        w->ent[ne].e = e;
        ++ne;
      }
      if (k == r->len) break;
      t = r->nb[k];
      e = r->cnt[k];
      old += encode_cost_for_pair(rep, si, t, (int64_t)o->sizes_by_rep[t], e);
      w->ent[ne].t = t;
      w->ent[ne].i = i;
      w->ent[ne].e = e;
      ++ne;
    }
    w->old[i] = old;
  }
  out->view_nnz = ne;
  const size_t gg = (size_t)g * (size_t)g;
  memset(w->pmat, 0, sizeof(int64_t) * gg);
  memset(w->fmat, 0, gg);
  qsort(w->ent, ne, sizeof(tentry), cmp_tentry);
  uint64_t examined = 0;
  for (size_t s = 0; s < ne;) {
    size_t e = s + 1;
    while (e < ne && w->ent[e].t == w->ent[s].t) ++e;
    if (e - s >= 2) {
      const int32_t t = w->ent[s].t;
      const int64_t st = (int64_t)o->sizes_by_rep[t];
      for (size_t x = s; x < e; ++x) {
        const int32_t ai = w->ent[x].i;
        const int32_t ra = q[ai];
        if (t == ra) continue;
        const int64_t sa = o->qsize[ra];
        const int64_t ea = w->ent[x].e;
        for (size_t y = x + 1; y < e; ++y) {
          const int32_t bi = w->ent[y].i;
          const int32_t rb = q[bi];
          if (t == rb) continue;
          ++examined;
          const int64_t sb = o->qsize[rb];
          const int64_t eb = w->ent[y].e;
          const int64_t oldc = encode_cost_for_pair(ra, sa, t, st, ea) + encode_cost_for_pair(rb, sb, t, st, eb);
          const int64_t newc = encode_cost_for_pair(ra, sa + sb, t, st, ea + eb);
          const int64_t delta = oldc - newc;
          if (delta <= 0) continue;
          w->pmat[(size_t)ai * (size_t)g + (size_t)bi] += delta;
        }
      }
    }
    s = e;
  }
  out->examined = examined;
  /* direct edges between members */
  for (int32_t i = 0; i < g; ++i) {
    w->map[i].rep = q[i];
    w->map[i].idx = i;
  }
  qsort(w->map, (size_t)g, sizeof(repidx), cmp_repidx);
  for (int32_t i = 0; i < g; ++i) {
    const qrow* r = &o->rows[q[i]];
    for (int32_t k = 0; k < r->len; ++k) {
      const int32_t j = find_idx(w->map, g, r->nb[k]);
      if (j < 0 || i >= j) continue;
      w->pmat[(size_t)i * (size_t)g + (size_t)j] += r->cnt[k];
    }
  }
  /* per-member top-k ranking */
  for (int32_t i = 0; i < g; ++i) {
    int32_t nr = 0;
    for (int32_t j = 0; j < g; ++j) {
      if (j == i) continue;
      const int32_t a = i < j ? i : j;
      const int32_t b = i < j ? j : i;
      const int64_t pg = w->pmat[(size_t)a * (size_t)g + (size_t)b];
      if (pg <= 0) continue;
      int64_t denom = w->old[a] + w->old[b];
      if (denom < 1) denom = 1;
      ranked* rk = &w->rk[nr++];
      rk->other = j;
      rk->pg = pg;
      rk->ratio = (double)pg / (double)denom;
      rk->lo = q[a] < q[b] ? q[a] : q[b];
      rk->hi = q[a] < q[b] ? q[b] : q[a];
    }
    if (nr == 0) continue;
    qsort(w->rk, (size_t)nr, sizeof(ranked), cmp_ranked);
    const int32_t keep = nr < top_k ? nr : top_k;
    for (int32_t p = 0; p < keep; ++p) {
      const int32_t j = w->rk[p].other;
      const int32_t a = i < j ? i : j;
      const int32_t b = i < j ? j : i;
      w->fmat[(size_t)a * (size_t)g + (size_t)b] = 1;
    }
  }
  int64_t nc = 0;
  for (size_t k = 0; k < gg; ++k) nc += w->fmat[k];
  out->c = (cand*)xmalloc(sizeof(cand) * (size_t)(nc > 0 ? nc : 1));
  int64_t p = 0;
  for (int32_t a = 0; a < g; ++a) {
    for (int32_t b = a + 1; b < g; ++b) {
      if (w->fmat[(size_t)a * (size_t)g + (size_t)b]) {
        out->c[p].a = a;
        out->c[p].b = b;
        out->c[p].gain = 0;
        out->c[p].before = 0;
        ++p;
      }
    }
  }
  out->nc = nc;
  return 0;
}

int64_t beam_oracle_prepare_group(beam_oracle* o, const int32_t* q, int32_t g, int32_t* a_idx,
                                  int32_t* b_idx, int64_t cap) {
  prepared pr;
  if (prepare_group(o, &o->ws[0], q, g, &pr) != 0) return -1;
  for (int64_t k = 0; k < pr.nc && k < cap; ++k) {
    a_idx[k] = pr.c[k].a;
    b_idx[k] = pr.c[k].b;
  }
  const int64_t nc = pr.nc;
  free(pr.c);
  return nc;
}

/* ----------------------------------------------- score, filter, select */

/* ScoreBatchEncodingAwarePreparedGroup -> ScoreCandidatesPersistentCpu
 * (src/sweg.cpp:2001-2129, src/scoring_cpu.cpp:67-116) followed by
 * FilterPreparedCandidatePairsByThreshold (src/sweg.cpp:2146-2186). */
static int score_and_filter(beam_oracle* o, prepared* pr, double threshold) {
  if (pr->nc == 0) return 0;
  o->st.merge_exact_gain_calls += (uint64_t)pr->nc;
  uint64_t input_nnz = 0;
  for (int64_t k = 0; k < pr->nc; ++k) {
    const int32_t ra = pr->q[pr->c[k].a], rb = pr->q[pr->c[k].b];
    input_nnz += (uint64_t)o->rows[ra].len + (o->qint[ra] > 0 ? 1u : 0u);
    input_nnz += (uint64_t)o->rows[rb].len + (o->qint[rb] > 0 ? 1u : 0u);
  }
  o->st.exact_gain_input_nnz += input_nnz;
  int failed = 0;
  uint64_t raw_a = 0, raw_b = 0, uni = 0, ovl = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : raw_a, raw_b, uni, ovl) reduction(| : failed) \
    num_threads(o->nthreads)
  for (int64_t k = 0; k < pr->nc; ++k) {
    gain_work wk = {0, 0, 0, 0};
    if (exact_gain(o, pr->q[pr->c[k].a], pr->q[pr->c[k].b], &pr->c[k].gain, &pr->c[k].before, &wk) != 0) {
      failed = 1;
    }
    raw_a += wk.raw_a;
    raw_b += wk.raw_b;
    uni += wk.uni;
    ovl += wk.ovl;
  }
  if (failed) {
    set_err("exact merge gain failed during scoring");
    return -1;
  }
  o->st.exact_raw_entries_a += raw_a;
  o->st.exact_raw_entries_b += raw_b;
  o->st.exact_union_neighbors += uni;
  o->st.exact_overlap_neighbors += ovl;
  int64_t kept = 0;
  for (int64_t k = 0; k < pr->nc; ++k) {
    const cand c = pr->c[k];
    const double ratio = c.before > 0 ? (double)c.gain / (double)c.before : 0.0;
    if (c.gain <= 0) {
      o->st.merge_rejected_by_threshold++;
      continue;
    }
    if (o->cfg.ea_use_threshold) {
      if (c.before <= 0 || ratio < threshold) {
        o->st.merge_rejected_by_threshold++;
        continue;
      }
    }
    o->st.merge_positive_gain_pairs++;
    pr->c[kept++] = c;
  }
  pr->nc = kept;
  return 0;
}

/* g0 order (src/sweg.cpp:2217-2235): gain desc, a_idx asc, b_idx asc. */
static int cmp_cand(const void* x, const void* y) {
  const cand* a = (const cand*)x;
  const cand* b = (const cand*)y;
  if (a->gain != b->gain) return a->gain > b->gain ? -1 : 1;
  if (a->a != b->a) return a->a < b->a ? -1 : 1;
  return a->b < b->b ? -1 : (a->b > b->b ? 1 : 0);
}

/* SelectScoredBatchEncodingAwareGroupPairs, g0 (src/sweg.cpp:2188-2281):
 * greedy endpoint-disjoint pass over the sorted pairs; emits (q[a], q[b]). */
static int64_t select_group(beam_oracle* o, prepared* pr, int32_t* out_keep, int32_t* out_remove,
                            int64_t* out_gain) {
  if (pr->g < 2 || pr->nc == 0) return 0;
  qsort(pr->c, (size_t)pr->nc, sizeof(cand), cmp_cand);
  uint8_t* used = (uint8_t*)xcalloc((size_t)pr->g, 1);
  int64_t ns = 0;
  int64_t total = 0;
  for (int64_t k = 0; k < pr->nc; ++k) {
    const cand c = pr->c[k];
    if (used[c.a] || used[c.b]) {
      o->st.merge_rejected_by_overlap++;
      continue;
    }
    if (o->I[pr->q[c.a]] == -1 || o->I[pr->q[c.b]] == -1) continue;
    used[c.a] = 1;
    used[c.b] = 1;
    out_keep[ns] = pr->q[c.a];
    out_remove[ns] = pr->q[c.b];
    out_gain[ns] = c.gain;
    total += c.gain;
    ++ns;
  }
  free(used);
  o->st.merge_candidate_pairs += pr->nc;
  o->st.merge_selected_pairs += ns;
  o->st.merge_total_local_gain += total;
  return ns;
}

/* CommitSelectedPairs, g0 (src/sweg.cpp:2665-2769): every selected pair is
 * validated with ExactMergeGainPersistent against the state at the start of
 * the commit (Update_S runs only after the validation loop), then the
 * accepted pairs are applied in order with Update_S. */
static int commit_pairs(beam_oracle* o, const int32_t* keep, const int32_t* remove, const int64_t* gains,
                        int64_t count) {
  uint8_t* ok = (uint8_t*)xcalloc((size_t)(count > 0 ? count : 1), 1);
  for (int64_t k = 0; k < count; ++k) {
    o->st.isolated_gain_sum += gains[k];
    o->st.selected_merges_for_validation++;
    if (o->I[keep[k]] == -1 || o->I[remove[k]] == -1) {
      o->st.stale_endpoint++;
      continue;
    }
    int64_t g = 0, b = 0;
    gain_work wk = {0, 0, 0, 0};
    if (exact_gain(o, keep[k], remove[k], &g, &b, &wk) != 0) {
      free(ok);
      set_err("exact merge gain failed during commit validation");
      return -1;
    }
    o->st.validation_exact_calls++;
    o->st.validation_exact_row_entry_work += wk.raw_a + wk.raw_b;
    if (g > 0) {
      ok[k] = 1;
    } else {
      o->st.rejected_nonpositive++;
    }
  }
  for (int64_t k = 0; k < count; ++k) {
    if (!ok[k]) continue;
    update_s(o, keep[k], remove[k]);
    o->st.accepted_merges_after_validation++;
  }
  free(ok);
  return 0;
}

/* Sweg::Merge, blocked mode (src/sweg.cpp:953-1145) with the reciprocal
 * threshold 1/(iter+1) (src/sweg.cpp:400-406), over the blocks that start at
 * group first_group, in order; stops after the block during which budget_ms
 * of wall time ran out (budget_ms <= 0: no limit). *next_group receives the
 * first group of the next unprocessed block. */
static int merge_blocks(beam_oracle* o, int iter, int64_t first_group, double budget_ms, int64_t* next_group) {
  const double threshold = 1.0 / (double)(iter + 1);
  const double start_ms = now_ms();
  const int64_t bs = o->cfg.group_batch_size;
  prepared* prep = (prepared*)xcalloc((size_t)bs, sizeof(prepared));
  int32_t* items = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)bs);
  int64_t sel_cap = 1024;
  int32_t* sk = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)sel_cap);
  int32_t* sr = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)sel_cap);
  int64_t* sg = (int64_t*)xmalloc(sizeof(int64_t) * (size_t)sel_cap);
  int rc = 0;
  int64_t b0 = first_group;
  for (; b0 < o->n_groups && rc == 0; b0 += bs) {
    if (budget_ms > 0 && b0 > first_group && now_ms() - start_ms >= budget_ms) break;
    const int64_t b1 = b0 + bs < o->n_groups ? b0 + bs : o->n_groups;
    int32_t nw = 0;
    for (int64_t gi = b0; gi < b1; ++gi) {
      if (o->glen[gi] >= 2) items[nw++] = (int32_t)gi;
    }
    const double t0 = now_ms();
    int failed = 0;
#pragma omp parallel for schedule(dynamic, 1) if (nw > 1) reduction(| : failed) num_threads(o->nthreads)
    for (int32_t wi = 0; wi < nw; ++wi) {
      const int32_t gi = items[wi];
      if (prepare_group(o, &o->ws[omp_get_thread_num()], o->reps + o->gstart[gi], o->glen[gi], &prep[wi]) != 0) {
        failed = 1;
      }
    }
    if (failed) {
      rc = -1;
      break;
    }
    o->st.merge_prepare_wall_ms += now_ms() - t0;
    for (int32_t wi = 0; wi < nw; ++wi) {
      const int32_t g = prep[wi].g;
      o->st.merge_group_count++;
      if ((uint64_t)g > o->st.merge_group_max_size) o->st.merge_group_max_size = (uint64_t)g;
      o->st.merge_raw_pair_count += (uint64_t)g * (uint64_t)(g - 1) / 2;
      o->st.merge_candidate_pairs_after_prune += (uint64_t)prep[wi].nc;
      o->st.candidate_proxy_pairs_examined += prep[wi].examined;
    }
    const double t1 = now_ms();
    for (int32_t wi = 0; wi < nw && rc == 0; ++wi) rc = score_and_filter(o, &prep[wi], threshold);
    if (rc != 0) break;
    const double t2 = now_ms();
    o->st.merge_gain_scoring_ms += t2 - t1;
    int64_t ns = 0;
    for (int32_t wi = 0; wi < nw; ++wi) {
      if (ns + prep[wi].g > sel_cap) {
        while (ns + prep[wi].g > sel_cap) sel_cap *= 2;
        sk = (int32_t*)realloc(sk, sizeof(int32_t) * (size_t)sel_cap);
        sr = (int32_t*)realloc(sr, sizeof(int32_t) * (size_t)sel_cap);
        sg = (int64_t*)realloc(sg, sizeof(int64_t) * (size_t)sel_cap);
      }
      ns += select_group(o, &prep[wi], sk + ns, sr + ns, sg + ns);
      free(prep[wi].c);
      prep[wi].c = NULL;
    }
    const double t3 = now_ms();
    o->st.merge_selection_ms += t3 - t2;
    rc = commit_pairs(o, sk, sr, sg, ns);
    o->st.merge_update_ms += now_ms() - t3;
  }
  free(prep);
  free(items);
  free(sk);
  free(sr);
  free(sg);
  if (next_group) *next_group = b0 < o->n_groups ? b0 : o->n_groups;
  return rc;
}

int beam_oracle_merge(beam_oracle* o, int iter, int total_iterations) {
  (void)total_iterations;
  return merge_blocks(o, iter, 0, 0.0, NULL);
}

int beam_oracle_merge_blocks(beam_oracle* o, int iter, int64_t first_group, double budget_ms,
                             int64_t* next_group) {
  if (first_group < 0 || first_group > o->n_groups || first_group % o->cfg.group_batch_size != 0) {
    set_err("first_group must be a block boundary within the iteration's groups");
    return -1;
  }
  return merge_blocks(o, iter, first_group, budget_ms, next_group);
}

/* Sweg::Run (src/sweg.cpp:651-709). */
int beam_oracle_run(beam_oracle* o, int iterations) {
  const double t0 = now_ms();
  for (int iter = 1; iter <= iterations; ++iter) {
    const double d0 = now_ms();
    if (beam_oracle_divide(o, iter) != 0) return -1;
    const double d1 = now_ms();
    o->st.runtime_divide_ms += d1 - d0;
    if (beam_oracle_merge(o, iter, iterations) != 0) return -1;
    o->st.runtime_merge_ms += now_ms() - d1;
  }
  o->st.runtime_run_ms = now_ms() - t0;
  uint64_t nnz = 0;
  for (int32_t r = 0; r < o->n; ++r) {
    if (o->qact[r]) nnz += (uint64_t)o->rows[r].len + (o->qint[r] > 0 ? 1u : 0u);
  }
  o->st.quotient_nnz_final = nnz;
  return 0;
}

/* ------------------------------------------------ partition views */

/* Sweg::CurrentPartitionLabels (src/sweg.cpp:2902-2918). */
int beam_oracle_labels(const beam_oracle* o, int32_t* labels) {
  for (int32_t i = 0; i < o->n; ++i) labels[i] = -1;
  for (int32_t rep = 0; rep < o->n; ++rep) {
    if (o->I[rep] == -1) continue;
    for (int32_t v = o->I[rep]; v != -1; v = o->J[v]) labels[v] = rep;
  }
  for (int32_t i = 0; i < o->n; ++i) {
    if (labels[i] < 0) {
      set_err("Partition contains an unlabeled node");
      return -1;
    }
  }
  return 0;
}

int beam_oracle_member_lists(const beam_oracle* o, int32_t* head, int32_t* next) {
  memcpy(head, o->I, sizeof(int32_t) * (size_t)o->n);
  memcpy(next, o->J, sizeof(int32_t) * (size_t)o->n);
  return 0;
}

/* Sweg::PartitionHash (src/sweg.cpp:2920-2928): FNV-1a over the labels. */
uint64_t beam_oracle_partition_hash(const beam_oracle* o) {
  int32_t* labels = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)o->n);
  if (beam_oracle_labels(o, labels) != 0) {
    free(labels);
    return 0;
  }
  uint64_t h = 1469598103934665603ULL;
  for (int32_t i = 0; i < o->n; ++i) {
    h ^= (uint64_t)(uint32_t)labels[i];
    h *= 1099511628211ULL;
  }
  free(labels);
  return h;
}

int beam_oracle_active(const beam_oracle* o, int32_t rep) { return o->qact[rep]; }
int64_t beam_oracle_size(const beam_oracle* o, int32_t rep) { return o->qsize[rep]; }
int64_t beam_oracle_internal(const beam_oracle* o, int32_t rep) { return o->qint[rep]; }

int64_t beam_oracle_row(const beam_oracle* o, int32_t rep, int32_t* nb, int64_t* cnt, int64_t cap) {
  const qrow* r = &o->rows[rep];
  for (int32_t k = 0; k < r->len && k < cap; ++k) {
    if (nb) nb[k] = r->nb[k];
    if (cnt) cnt[k] = r->cnt[k];
  }
  return r->len;
}

void beam_oracle_get_stats(const beam_oracle* o, beam_oracle_stats* out) { *out = o->st; }

/* CostOracle::ExactPartitionCost (src/cost_oracle.cpp:112-124): per pair of
 * labels the edge count between them, summed BlockCost; pairs are counted by
 * sorting packed label keys instead of a hash map. */
int64_t beam_oracle_exact_partition_cost(const beam_oracle* o) {
  int32_t* labels = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)o->n);
  if (beam_oracle_labels(o, labels) != 0) {
    free(labels);
    return -1;
  }
  int64_t* sizes = (int64_t*)xcalloc((size_t)o->n, sizeof(int64_t));
  for (int32_t v = 0; v < o->n; ++v) sizes[labels[v]]++;
  int64_t* keys = (int64_t*)xmalloc(sizeof(int64_t) * (size_t)(o->arcs / 2 + 1));
  int64_t nk = 0;
  for (int32_t u = 0; u < o->n; ++u) {
    for (int64_t k = o->row_ptr[u]; k < o->row_ptr[u + 1]; ++k) {
      const int32_t v = o->col[k];
      if (u < v) {
        const uint32_t a = (uint32_t)labels[u], b = (uint32_t)labels[v];
        const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
        keys[nk++] = (int64_t)(((uint64_t)lo << 32) | hi);
      }
    }
  }
  qsort(keys, (size_t)nk, sizeof(int64_t), cmp_i64);
  int64_t total = 0;
  int err = 0;
  for (int64_t s = 0; s < nk;) {
    int64_t e = s + 1;
    while (e < nk && keys[e] == keys[s]) ++e;
    const int32_t a = (int32_t)((uint64_t)keys[s] >> 32);
    const int32_t b = (int32_t)((uint64_t)keys[s] & 0xffffffffu);
    total += block_cost(sizes[a], sizes[b], e - s, a == b, &err);
    s = e;
  }
  free(keys);
  free(sizes);
  free(labels);
  if (err) {
    set_err("partition cost overflow");
    return -1;
  }
  return total;
}

/* -------------------------------------------------------- encode */

typedef struct {
  uint64_t key;
  int32_t u, v;
} pair_arc;

static int cmp_pair_arc(const void* x, const void* y) {
  const pair_arc* a = (const pair_arc*)x;
  const pair_arc* b = (const pair_arc*)y;
  if (a->key != b->key) return a->key < b->key ? -1 : 1;
  if (a->u != b->u) return a->u < b->u ? -1 : 1;
  return a->v < b->v ? -1 : (a->v > b->v ? 1 : 0);
}

typedef struct {
  int32_t a, b;
} epair;

static int cmp_epair(const void* x, const void* y) {
  const epair* a = (const epair*)x;
  const epair* b = (const epair*)y;
  if (a->a != b->a) return a->a < b->a ? -1 : 1;
  return a->b < b->b ? -1 : (a->b > b->b ? 1 : 0);
}

typedef struct {
  epair* e;
  int64_t n, cap;
} evec;

static void evec_push(evec* v, int32_t a, int32_t b) {
  if (v->n == v->cap) {
    v->cap = v->cap ? v->cap * 2 : 1024;
    v->e = (epair*)realloc(v->e, sizeof(epair) * (size_t)v->cap);
    if (!v->e) abort();
  }
  v->e[v->n].a = a;
  v->e[v->n].b = b;
  v->n++;
}

static int write_pairs(const char* dir, const char* name, const evec* v) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE* f = fopen(path, "w");
  if (!f) return -1;
  for (int64_t k = 0; k < v->n; ++k) fprintf(f, "%d\t%d\n", v->e[k].a, v->e[k].b);
  fclose(f);
  return 0;
}

/* Sweg::Encode, mags-compatible branch (src/sweg.cpp:3017-3163): supernodes
 * renumbered in rep order, arcs grouped by supernode pair (internal edges
 * once), sparse blocks (e <= 1 + cap - e) go to Cp, dense ones to P plus the
 * missing member pairs in Cm; all three lists sorted. Metrics follow
 * ComputeCompressionMetrics (include/compression_metrics.hpp:39-98). */
int beam_oracle_encode(beam_oracle* o, const char* dir, beam_oracle_encoding* out) {
  const int32_t n = o->n;
  int32_t* new_id = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  int32_t* nts = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  int32_t* ssize = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  int32_t* shead = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)n);
  int32_t ns = 0;
  for (int32_t rep = 0; rep < n; ++rep) {
    if (o->I[rep] == -1) continue;
    int32_t cnt = 0;
    for (int32_t v = o->I[rep]; v != -1; v = o->J[v]) {
      nts[v] = ns;
      ++cnt;
    }
    new_id[ns] = rep;
    ssize[ns] = cnt;
    shead[ns] = o->I[rep];
    ++ns;
  }
  pair_arc* pa = (pair_arc*)xmalloc(sizeof(pair_arc) * (size_t)(o->arcs > 0 ? o->arcs : 1));
  int64_t np = 0;
  for (int32_t u = 0; u < n; ++u) {
    const int32_t su = nts[u];
    for (int64_t k = o->row_ptr[u]; k < o->row_ptr[u + 1]; ++k) {
      const int32_t v = o->col[k];
      const int32_t sv = nts[v];
      if (su > sv) continue;
      if (su == sv && u >= v) continue;
      pa[np].key = ((uint64_t)(uint32_t)su << 32) | (uint32_t)sv;
      pa[np].u = u;
      pa[np].v = v;
      ++np;
    }
  }
  qsort(pa, (size_t)np, sizeof(pair_arc), cmp_pair_arc);
  evec P = {0}, Cp = {0}, Cm = {0};
  for (int64_t s = 0; s < np;) {
    int64_t e = s + 1;
    while (e < np && pa[e].key == pa[s].key) ++e;
    const int32_t A = (int32_t)(pa[s].key >> 32);
    const int32_t B = (int32_t)(pa[s].key & 0xffffffffu);
    const int64_t real = e - s;
    const int64_t sa = ssize[A], sb = ssize[B];
    const int64_t cap = A == B ? sa * (sa - 1) / 2 : sa * sb;
    if (real <= 1 + cap - real) {
      for (int64_t k = s; k < e; ++k) evec_push(&Cp, pa[k].u, pa[k].v);
      s = e;
      continue;
    }
    evec_push(&P, A, B);
    /* block arcs are sorted by (u, v): binary-search membership */
    for (int32_t u = shead[A]; u != -1; u = o->J[u]) {
      for (int32_t v = shead[B]; v != -1; v = o->J[v]) {
        if (A == B && u >= v) continue;
        int64_t lo = s, hi = e;
        while (lo < hi) {
          const int64_t mid = lo + (hi - lo) / 2;
          if (pa[mid].u < u || (pa[mid].u == u && pa[mid].v < v)) lo = mid + 1; else hi = mid;
        }
        if (!(lo < e && pa[lo].u == u && pa[lo].v == v)) evec_push(&Cm, u, v);
      }
    }
    s = e;
  }
  qsort(P.e, (size_t)P.n, sizeof(epair), cmp_epair);
  qsort(Cp.e, (size_t)Cp.n, sizeof(epair), cmp_epair);
  qsort(Cm.e, (size_t)Cm.n, sizeof(epair), cmp_epair);
  int rc = 0;
  if (dir) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/G.txt", dir);
    FILE* f = fopen(path, "w");
    if (!f) {
      rc = -1;
    } else {
      for (int32_t sid = 0; sid < ns; ++sid) {
        fprintf(f, "%d", sid);
        for (int32_t v = shead[sid]; v != -1; v = o->J[v]) fprintf(f, "\t%d", v);
        fprintf(f, "\n");
      }
      fclose(f);
    }
    if (rc == 0) rc = write_pairs(dir, "P.txt", &P);
    if (rc == 0) rc = write_pairs(dir, "Cp.txt", &Cp);
    if (rc == 0) rc = write_pairs(dir, "Cm.txt", &Cm);
    if (rc != 0) set_err("Failed to write output files");
  }
  if (out) {
    out->n_supernodes = ns;
    out->p = P.n;
    out->cp = Cp.n;
    out->cm = Cm.n;
    int64_t loops = 0;
    for (int64_t k = 0; k < P.n; ++k) loops += P.e[k].a == P.e[k].b;
    out->num_superedges_loop = loops;
    out->num_superedges_nonloop = P.n - loops;
    out->encoding_cost_mags_x2 = 2 * (P.n + Cp.n + Cm.n);
    const int64_t m = o->arcs / 2;
    out->cost_ratio_mags_compatible = m > 0 ? (double)out->encoding_cost_mags_x2 / (2.0 * (double)m) : 0.0;
  }
  free(P.e);
  free(Cp.e);
  free(Cm.e);
  free(pa);
  free(new_id);
  free(nts);
  free(ssize);
  free(shead);
  return rc;
}

/* ------------------------------------------- legacy-objective flat scoring */

static int64_t legacy_cost(int32_t row_rep, int64_t row_size, int32_t nb_rep, int64_t nb_size, int64_t e) {
  const int64_t cap = row_rep == nb_rep ? row_size * (row_size - 1) / 2 : row_size * nb_size;
  const int64_t alt = 1 + cap - e;
  return e < alt ? e : alt;
}

typedef struct {
  int32_t ra, rb;
  int64_t sa, sb, la, lb;
  int64_t before, after;
  int seen_a, seen_b;
} legacy_acc;

static void legacy_term(legacy_acc* g, int32_t x, int64_t sx, int64_t ea_raw, int64_t eb_raw) {
  if (x == g->ra) g->seen_a = 1;
  if (x == g->rb) g->seen_b = 1;
  int64_t ea = ea_raw, eb = eb_raw;
  if (x == g->ra) ea = ea_raw > g->la ? ea_raw - g->la : 0;
  if (x == g->rb) eb = eb_raw > g->lb ? eb_raw - g->lb : 0;
  g->before += legacy_cost(g->ra, g->sa, x, sx, ea) + legacy_cost(g->rb, g->sb, x, sx, eb);
  const int64_t sm = g->sa + g->sb;
  g->after += legacy_cost(g->ra, sm, x == g->rb ? g->ra : x, x == g->rb ? sm : sx, ea + eb);
}

/* Legacy local gain of rows a and b of a flat per-block CSR, the host check
 * of the reference's CUDA mode (ComputeLocalGainHostFromFlat,
 * src/cuda_scoring.cu:146-252): a two-pointer union of the two sorted rows;
 * every neighbour x adds the costs of (a, x) and (b, x) before and of
 * (a+b, x) after, counts toward a row's own representative less its
 * self-loops, and a representative missing from both rows is added with
 * count 0. */
int beam_oracle_legacy_flat_gain(const int32_t* offsets, const int32_t* reps, const int64_t* row_sizes,
                                 const int64_t* self_loops, const int32_t* nb, const int64_t* wt,
                                 const int64_t* nsz, int32_t a, int32_t b, int64_t* gain, int64_t* before) {
  legacy_acc g = {reps[a], reps[b], row_sizes[a], row_sizes[b], self_loops[a], self_loops[b], 0, 0, 0, 0};
  int32_t ia = offsets[a], ib = offsets[b];
  const int32_t ea = offsets[a + 1], eb = offsets[b + 1];
  while (ia < ea || ib < eb) {
    if (ib >= eb || (ia < ea && nb[ia] < nb[ib])) {
      legacy_term(&g, nb[ia], nsz[ia], wt[ia], 0);
      ++ia;
    } else if (ia >= ea || nb[ib] < nb[ia]) {
      legacy_term(&g, nb[ib], nsz[ib], 0, wt[ib]);
      ++ib;
    } else {
      legacy_term(&g, nb[ia], nsz[ia], wt[ia], wt[ib]);
      ++ia;
      ++ib;
    }
  }
  if (!g.seen_a) legacy_term(&g, g.ra, g.sa, 0, 0);
  if (g.rb != g.ra && !g.seen_b) legacy_term(&g, g.rb, g.sb, 0, 0);
  *gain = g.before - g.after;
  *before = g.before;
  return 0;
}
