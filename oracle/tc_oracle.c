/*
 * tc_oracle.c — CPU oracle for the triangle-counting path.  TEST INFRASTRUCTURE ONLY.
 *
 * Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs load this
 * library, and only as the checker.  The product (trust_gb300/) never links or calls it.
 *
 * Contents, each a plain restatement of the reference's algorithm:
 *   orc_count_forward      forward-intersection counter with the counted quantity of
 *                          dynamic_assign (Without-graph-partition/TC.cu:230-600); the merge
 *                          step follows Without-graph-partition/graph.hpp:133-149
 *   orc_trust_check        decides whether the reference kernel is exact on a CSR: bucket loads
 *                          vs BUCKET_SIZE=100 (TC.cu:16, :285-302), the bin+1 re-probe at >=99
 *                          entries (TC.cu:105-107), the d<2 early exit (TC.cu:440) and the
 *                          degree-split binary search (TC.cu:191-205, :632)
 *   orc_ref_undirect       Preprocess/fromDirectToUndirect.cpp:53-119 (selectVertex/deleteedge)
 *   orc_ref_outdegree_csr  Preprocess/preprocess_outdegree.cpp:42-253; std::sort tie order is
 *                          replaced by a stable order (the triangle count does not depend on it)
 *   orc_build_csr          the synthetic-config pipeline: drop self-loops, symmetrise, dedupe,
 *                          drop orphans, orient low->high (degree, id), renumber by out-degree
 *                          descending (ties by id), rows sorted
 *   orc_partition          Preprocess/partition.cpp:72-121 tile split
 *   orc_gen_*              CPU twins of the counter-based graph generators
 *
 * Parity pins: the reference preprocess binaries built from source (oracle/build_ref.sh) give
 * golden CSRs under tests/golden/; analytic counts (K_n, grids, stars, bipartite) pin the
 * counter.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t i64;
typedef int32_t i32;
typedef uint64_t u64;

/* ------------------------------------------------------------------------------------------ */
/* sorting helpers                                                                             */
/* ------------------------------------------------------------------------------------------ */
static int cmp_i32(const void *a, const void *b) {
  i32 x = *(const i32 *)a, y = *(const i32 *)b;
  return (x > y) - (x < y);
}
static int cmp_u64(const void *a, const void *b) {
  u64 x = *(const u64 *)a, y = *(const u64 *)b;
  return (x > y) - (x < y);
}

/* LSD radix sort of u64 keys (8-bit digits over the low `bits` bits); stable. */
static int radix_u64(u64 *a, i64 n, int bits) {
  u64 *tmp = (u64 *)malloc(sizeof(u64) * (size_t)(n > 0 ? n : 1));
  if (!tmp) return -1;
  u64 *src = a, *dst = tmp;
  for (int sh = 0; sh < bits; sh += 8) {
    i64 cnt[257];
    memset(cnt, 0, sizeof cnt);
    for (i64 i = 0; i < n; ++i) cnt[((src[i] >> sh) & 255) + 1]++;
    for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
    for (i64 i = 0; i < n; ++i) dst[cnt[(src[i] >> sh) & 255]++] = src[i];
    u64 *t = src; src = dst; dst = t;
  }
  if (src != a) memcpy(a, src, sizeof(u64) * (size_t)n);
  free(tmp);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* the counted quantity                                                                        */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
  const i64 *beg;
  const i32 *adj;
  const i32 *sorted; /* per-row sorted copy of adj */
  i64 lo, n;         /* source vertices [lo, n) */
  i64 stride;        /* every stride-th of them: lo, lo + stride, ... */
  int min_deg;
  atomic_llong next;
  atomic_ullong total;
} count_job;

/* |set(row v) ∩ row u| with multiplicity on the row-u side: merge of the sorted rows
 * (Without-graph-partition/graph.hpp:133-149 merges two sorted lists the same way). */
static u64 merge_count(const i32 *a, i64 na, const i32 *b, i64 nb) {
  u64 c = 0;
  i64 i = 0, j = 0;
  while (i < na && j < nb) {
    if (a[i] < b[j]) {
      ++i;
    } else if (a[i] > b[j]) {
      ++j;
    } else {
      i32 x = a[i];
      while (j < nb && b[j] == x) { ++c; ++j; }
      while (i < na && a[i] == x) ++i;
    }
  }
  return c;
}

static void *count_worker(void *arg) {
  count_job *J = (count_job *)arg;
  const i64 CH = 256;
  u64 local = 0;
  const i64 samples = (J->n - J->lo + J->stride - 1) / J->stride;
  for (;;) {
    i64 k0 = atomic_fetch_add(&J->next, CH);
    if (k0 >= samples) break;
    i64 k1 = k0 + CH < samples ? k0 + CH : samples;
    for (i64 k = k0; k < k1; ++k) {
      const i64 v = J->lo + k * J->stride;
      i64 b = J->beg[v], e = J->beg[v + 1];
      if (e - b < J->min_deg) continue;
      const i32 *rv = J->sorted + b;
      for (i64 i = b; i < e; ++i) {
        i32 u = J->adj[i];
        local += merge_count(rv, e - b, J->sorted + J->beg[u], J->beg[u + 1] - J->beg[u]);
      }
    }
  }
  atomic_fetch_add(&J->total, local);
  return NULL;
}

static void run_count(const i64 *beg, const i32 *adj, const i32 *sorted, i64 lo, i64 hi, i64 stride, int min_deg,
                      int threads, u64 *out) {
  count_job J;
  J.beg = beg; J.adj = adj; J.sorted = sorted; J.lo = lo; J.n = hi; J.stride = stride; J.min_deg = min_deg;
  atomic_init(&J.next, 0);
  atomic_init(&J.total, 0);
  if (threads <= 1) {
    count_worker(&J);
  } else {
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
    int started = 0;
    for (int t = 0; t < threads; ++t)
      if (pthread_create(&th[t], NULL, count_worker, &J) == 0) ++started;
    if (started == 0) count_worker(&J);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
  }
  *out = (u64)atomic_load(&J.total);
}

/* Sum over v with d(v) >= min_deg, over arcs (v,u), over arcs (u,w), of [w in row v].
 * threads <= 0 uses one thread.  Returns 0 on success. */
int orc_count_forward(const i64 *beg, const i32 *adj, i64 n, int min_deg, int threads, u64 *out) {
  i64 m = beg[n];
  i32 *sorted = (i32 *)malloc(sizeof(i32) * (size_t)(m > 0 ? m : 1));
  if (!sorted) return -1;
  memcpy(sorted, adj, sizeof(i32) * (size_t)m);
  for (i64 v = 0; v < n; ++v)
    if (beg[v + 1] - beg[v] > 1) qsort(sorted + beg[v], (size_t)(beg[v + 1] - beg[v]), sizeof(i32), cmp_i32);
  *out = 0;
  run_count(beg, adj, sorted, 0, n, 1, min_deg, threads, out);
  free(sorted);
  return 0;
}

/* Same quantity restricted to source vertices [lo, hi), on a CSR whose rows are already sorted
 * ascending (no per-row sort inside): the bounded CPU-baseline sample. */
int orc_count_forward_sorted_range(const i64 *beg, const i32 *adj, i64 n, i64 lo, i64 hi, int min_deg,
                                   int threads, u64 *out) {
  if (lo < 0) lo = 0;
  if (hi > n) hi = n;
  *out = 0;
  if (lo >= hi) return 0;
  run_count(beg, adj, adj, lo, hi, 1, min_deg, threads, out);
  return 0;
}

/* The same quantity over the source vertices start, start + stride, ... < n of a CSR with sorted
 * rows: a systematic sample of rows of every degree class (the bounded CPU-baseline sample on
 * graphs whose whole count takes minutes).  *arcs receives the sampled vertices' arc count. */
int orc_count_forward_stride(const i64 *beg, const i32 *adj, i64 n, i64 start, i64 stride, int min_deg, int threads,
                             u64 *out, u64 *arcs) {
  *out = 0;
  *arcs = 0;
  if (stride < 1 || start < 0) return -1;
  if (start >= n) return 0;
  u64 a = 0;
  for (i64 v = start; v < n; v += stride)
    if (beg[v + 1] - beg[v] >= min_deg) a += (u64)(beg[v + 1] - beg[v]);
  *arcs = a;
  run_count(beg, adj, adj, start, n, stride, min_deg, threads, out);
  return 0;
}

/* Wedge count W = sum over arcs (v,u) with d(v) >= min_deg of d(u) (the probe count). */
u64 orc_wedges(const i64 *beg, const i32 *adj, i64 n, int min_deg) {
  u64 w = 0;
  for (i64 v = 0; v < n; ++v) {
    if (beg[v + 1] - beg[v] < min_deg) continue;
    for (i64 i = beg[v]; i < beg[v + 1]; ++i) w += (u64)(beg[adj[i] + 1] - beg[adj[i]]);
  }
  return w;
}

/* Tile-job form used by the partitioned path: rows r of A (tables) and B (arcs), probing rows of
 * C.  Counts sum_r [dA>=1 && dB>=1] sum_{u in B[r]} |set(A[r]) ∩ C[u]|. */
int orc_count_tiles(const i64 *begA, const i32 *adjA, const i64 *begB, const i32 *adjB,
                    const i64 *begC, const i32 *adjC, i64 rows, i64 rowsC, u64 *out) {
  i64 mA = begA[rows], mC = begC[rowsC];
  i32 *sA = (i32 *)malloc(sizeof(i32) * (size_t)(mA > 0 ? mA : 1));
  i32 *sC = (i32 *)malloc(sizeof(i32) * (size_t)(mC > 0 ? mC : 1));
  if (!sA || !sC) { free(sA); free(sC); return -1; }
  memcpy(sA, adjA, sizeof(i32) * (size_t)mA);
  memcpy(sC, adjC, sizeof(i32) * (size_t)mC);
  for (i64 r = 0; r < rows; ++r) qsort(sA + begA[r], (size_t)(begA[r + 1] - begA[r]), sizeof(i32), cmp_i32);
  for (i64 r = 0; r < rowsC; ++r) qsort(sC + begC[r], (size_t)(begC[r + 1] - begC[r]), sizeof(i32), cmp_i32);
  u64 total = 0;
  for (i64 r = 0; r < rows; ++r) {
    i64 dA = begA[r + 1] - begA[r], dB = begB[r + 1] - begB[r];
    if (dA < 1 || dB < 1) continue;
    for (i64 i = begB[r]; i < begB[r + 1]; ++i) {
      i32 u = adjB[i];
      total += merge_count(sA + begA[r], dA, sC + begC[u], begC[u + 1] - begC[u]);
    }
  }
  *out = total;
  free(sA);
  free(sC);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* validity of the reference kernel on a CSR                                                   */
/* ------------------------------------------------------------------------------------------ */
enum {
  ORC_TRUST_EXACT = 0,
  ORC_TRUST_BUCKET_OVERFLOW = 1, /* a bucket gets > 100 entries: entries dropped (TC.cu:299)   */
  ORC_TRUST_REPROBE = 2,         /* a bucket gets >= 99 entries: bin+1 scanned (TC.cu:105-107) */
  ORC_TRUST_EARLY_EXIT = 4,      /* a d<2 vertex precedes d>=2 vertices in the warp range      */
  ORC_TRUST_INT32 = 8            /* an offset >= 2^31 (TC.cu narrows to int, :267-268)         */
};

/* Without-graph-partition/TC.cu:191-205: last vertex whose out-degree exceeds val (binary search
 * that assumes the predicate is monotone). */
i64 orc_trust_split(const i64 *beg, i64 n, int val) {
  i64 l = 0, r = n;
  while (l < r - 1) {
    i64 mid = (l + r) / 2;
    if (beg[mid + 1] - beg[mid] > val) l = mid; else r = mid;
  }
  if (n == 0 || beg[l + 1] - beg[l] <= val) return -1;
  return l;
}

int orc_trust_check(const i64 *beg, const i32 *adj, i64 n, i64 *warpfirst_out) {
  int flags = 0;
  if (beg[n] >= ((i64)1 << 31)) flags |= ORC_TRUST_INT32;
  i64 warpfirst = orc_trust_split(beg, n, 100) + 1; /* TC.cu:632, USE_CTA = 100 */
  if (warpfirst_out) *warpfirst_out = warpfirst;
  int cnt[1024];
  for (i64 v = 0; v < n; ++v) {
    int nb = v < warpfirst ? 1024 : 32; /* block_bucketnum / warp_bucketnum, TC.cu:24-25 */
    i64 b = beg[v], e = beg[v + 1];
    if (v >= warpfirst && e - b < 2) continue;
    memset(cnt, 0, sizeof(int) * (size_t)nb);
    for (i64 i = b; i < e; ++i) {
      int k = ++cnt[adj[i] & (nb - 1)];
      if (k > 100) flags |= ORC_TRUST_BUCKET_OVERFLOW;
      if (k >= 99) flags |= ORC_TRUST_REPROBE;
    }
  }
  /* warp loop ends at the first d<2 vertex a warp meets (TC.cu:440): every d>=2 vertex of the
   * warp range must come before every d<2 vertex */
  int seen_small = 0;
  for (i64 v = warpfirst; v < n; ++v) {
    i64 d = beg[v + 1] - beg[v];
    if (d < 2) seen_small = 1;
    else if (seen_small) { flags |= ORC_TRUST_EARLY_EXIT; break; }
  }
  return flags;
}

/* ------------------------------------------------------------------------------------------ */
/* the synthetic-config pipeline (the product's GPU preprocessing must match it byte for byte) */
/* ------------------------------------------------------------------------------------------ */
/* pairs: 2*np ints (u at even index), ids in [0, id_bound).  Outputs malloc'd. */
int orc_build_csr(const i32 *pairs, i64 np, i64 id_bound, i64 **beg_out, i32 **adj_out, i64 *n_out,
                  i64 *m_out) {
  int idbits = 1;
  while (((i64)1 << idbits) <= id_bound) ++idbits;
  u64 *e = (u64 *)malloc(sizeof(u64) * (size_t)(np > 0 ? np : 1));
  if (!e) return -1;
  i64 ne = 0;
  for (i64 i = 0; i < np; ++i) {
    u64 u = (u64)(uint32_t)pairs[2 * i], v = (u64)(uint32_t)pairs[2 * i + 1];
    if (u == v) continue;
    u64 a = u < v ? u : v, b = u < v ? v : u;
    e[ne++] = (a << 32) | b;
  }
  if (radix_u64(e, ne, 32 + idbits)) { free(e); return -1; }
  i64 nu = 0;
  for (i64 i = 0; i < ne; ++i)
    if (i == 0 || e[i] != e[i - 1]) e[nu++] = e[i];
  i64 *deg = (i64 *)calloc((size_t)(id_bound > 0 ? id_bound : 1), sizeof(i64));
  i64 *cid = (i64 *)malloc(sizeof(i64) * (size_t)(id_bound > 0 ? id_bound : 1));
  for (i64 i = 0; i < nu; ++i) { deg[e[i] >> 32]++; deg[e[i] & 0xffffffffu]++; }
  i64 n = 0;
  for (i64 x = 0; x < id_bound; ++x) cid[x] = deg[x] > 0 ? n++ : -1;
  /* orientation order: (degree, compacted id) ascending */
  u64 *ord = (u64 *)malloc(sizeof(u64) * (size_t)(n > 0 ? n : 1));
  i64 *pos = (i64 *)malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
  i64 *cdeg = (i64 *)malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
  for (i64 x = 0; x < id_bound; ++x) if (cid[x] >= 0) cdeg[cid[x]] = deg[x];
  for (i64 c = 0; c < n; ++c) ord[c] = ((u64)cdeg[c] << 32) | (u64)c;
  qsort(ord, (size_t)n, sizeof(u64), cmp_u64);
  for (i64 p = 0; p < n; ++p) pos[ord[p] & 0xffffffffu] = p;
  /* orient and count out-degrees */
  i64 *od = (i64 *)calloc((size_t)(n > 0 ? n : 1), sizeof(i64));
  for (i64 i = 0; i < nu; ++i) {
    i64 a = cid[e[i] >> 32], b = cid[e[i] & 0xffffffffu];
    i64 src = pos[a] < pos[b] ? a : b, dst = pos[a] < pos[b] ? b : a;
    e[i] = ((u64)src << 32) | (u64)dst;
    od[src]++;
  }
  /* renumber: out-degree descending, ties by compacted id */
  for (i64 c = 0; c < n; ++c) ord[c] = ((u64)(0xffffffffu - (uint32_t)od[c]) << 32) | (u64)c;
  qsort(ord, (size_t)n, sizeof(u64), cmp_u64);
  i64 *newid = pos; /* reuse */
  for (i64 p = 0; p < n; ++p) newid[ord[p] & 0xffffffffu] = p;
  for (i64 i = 0; i < nu; ++i) {
    i64 s = newid[e[i] >> 32], d = newid[e[i] & 0xffffffffu];
    e[i] = ((u64)s << 32) | (u64)d;
  }
  int nbits = 1;
  while (((i64)1 << nbits) <= n) ++nbits;
  radix_u64(e, nu, 32 + nbits);
  i64 *beg = (i64 *)calloc((size_t)(n + 1), sizeof(i64));
  i32 *adj = (i32 *)malloc(sizeof(i32) * (size_t)(nu > 0 ? nu : 1));
  for (i64 i = 0; i < nu; ++i) { beg[(e[i] >> 32) + 1]++; adj[i] = (i32)(e[i] & 0xffffffffu); }
  for (i64 v = 0; v < n; ++v) beg[v + 1] += beg[v];
  free(e); free(deg); free(cid); free(ord); free(pos); free(cdeg); free(od);
  *beg_out = beg; *adj_out = adj; *n_out = n; *m_out = nu;
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* reference preprocessing, restated                                                           */
/* ------------------------------------------------------------------------------------------ */
/* Preprocess/fromDirectToUndirect.cpp:53-119.  Input: np pairs of ids >= 0.  Vertices that
 * appear are renumbered 1..k in increasing id order; each pair becomes (min,max); per-min
 * duplicates are removed.  Output: k, and the edge list sorted by (u, v), 1-based, self-loops
 * kept (u == v).  out must hold 2*np ints. */
int orc_ref_undirect(const i32 *pairs, i64 np, i64 *k_out, i32 *out, i64 *m_out) {
  i32 maxv = 0;
  for (i64 i = 0; i < 2 * np; ++i) if (pairs[i] > maxv) maxv = pairs[i];
  i32 *a = (i32 *)calloc((size_t)maxv + 2, sizeof(i32));
  for (i64 i = 0; i < 2 * np; ++i) a[pairs[i]] = 1;
  i32 k = 0;
  for (i32 x = 0; x <= maxv; ++x) if (a[x]) a[x] = ++k;
  u64 *e = (u64 *)malloc(sizeof(u64) * (size_t)(np > 0 ? np : 1));
  for (i64 i = 0; i < np; ++i) {
    u64 u = (u64)a[pairs[2 * i]], v = (u64)a[pairs[2 * i + 1]];
    if (u > v) { u64 t = u; u = v; v = t; }
    e[i] = (u << 32) | v;
  }
  qsort(e, (size_t)np, sizeof(u64), cmp_u64);
  i64 m = 0;
  for (i64 i = 0; i < np; ++i) {
    if (i && e[i] == e[i - 1]) continue;
    out[2 * m] = (i32)(e[i] >> 32);
    out[2 * m + 1] = (i32)(e[i] & 0xffffffffu);
    ++m;
  }
  free(a); free(e);
  *k_out = k; *m_out = m;
  return 0;
}

typedef struct {
  i32 id;     /* vertexID */
  i32 newid;
  i64 len, cap;
  i32 *e;
} orc_vtx;

static void vpush(orc_vtx *v, i32 x) {
  if (v->len == v->cap) {
    v->cap = v->cap ? 2 * v->cap : 4;
    v->e = (i32 *)realloc(v->e, sizeof(i32) * (size_t)v->cap);
  }
  v->e[v->len++] = x;
}

static int g_cmp_dir;
static int cmp_vtx_len(const void *pa, const void *pb) {
  const orc_vtx *a = (const orc_vtx *)pa, *b = (const orc_vtx *)pb;
  if (a->len != b->len) return g_cmp_dir * ((a->len > b->len) - (a->len < b->len));
  /* stable stand-in for std::sort's unspecified tie order: keep the current order */
  return (a->newid > b->newid) - (a->newid < b->newid);
}

static void sort_by_len(orc_vtx *V, i64 n, int dir) {
  for (i64 i = 0; i < n; ++i) V[i].newid = (i32)i; /* current position as the tie key */
  g_cmp_dir = dir;
  qsort(V, (size_t)n, sizeof(orc_vtx), cmp_vtx_len);
}

/* Preprocess/preprocess_outdegree.cpp:42-253 on a 1-based undirected edge list (the output of
 * orc_ref_undirect).  Writes begin (k+1 int64) and adjacent (int32) like computeCSR (:186-222).
 * s2/s3 receive the class boundaries of reassignID (:100-113). */
int orc_ref_outdegree_csr(i64 k, const i32 *edges, i64 m, i64 *beg, i32 *adj, i64 *s2_out, i64 *s3_out) {
  i64 n = k;
  orc_vtx *V = (orc_vtx *)calloc((size_t)(n > 0 ? n : 1), sizeof(orc_vtx));
  for (i64 i = 0; i < n; ++i) V[i].id = (i32)i;
  for (i64 i = 0; i < m; ++i) { /* loadgraph :71-76 */
    i32 u = edges[2 * i] - 1, v = edges[2 * i + 1] - 1;
    vpush(&V[u], v);
    vpush(&V[v], u);
  }
  sort_by_len(V, n, +1); /* :226 degree ascending */
  /* orientation :79-98 — keep w with position(w) > i, in reverse list order */
  i32 *a = (i32 *)malloc(sizeof(i32) * (size_t)(n > 0 ? n : 1));
  for (i64 i = 0; i < n; ++i) a[V[i].id] = (i32)i;
  for (i64 i = 0; i < n; ++i) {
    i32 *x = V[i].e;
    i64 len = V[i].len;
    V[i].e = NULL; V[i].len = 0; V[i].cap = 0;
    for (i64 j = len - 1; j >= 0; --j) if (a[x[j]] > i) vpush(&V[i], x[j]);
    free(x);
  }
  sort_by_len(V, n, -1); /* :236 out-degree descending */
  /* computeCSR :188-200 — ids become positions */
  for (i64 i = 0; i < n; ++i) a[V[i].id] = (i32)i;
  for (i64 i = 0; i < n; ++i) {
    for (i64 j = 0; j < V[i].len; ++j) V[i].e[j] = a[V[i].e[j]];
    V[i].id = (i32)i;
  }
  /* reassignID :100-185 */
  i64 k1 = 0, k2 = -1, k3 = -1;
  for (i64 i = 0; i < n; ++i) {
    V[i].newid = -1;
    if (k2 == -1 && V[i].len <= 100) k2 = i;
    if (k3 == -1 && V[i].len < 2) k3 = i;
  }
  i64 s2 = k2, s3 = k3;
  for (i64 i = 0; i < n; ++i) {
    if (V[i].len <= 2) break;
    for (i64 j = 0; j < V[i].len; ++j) {
      i32 v = V[i].e[j];
      if (V[v].newid == -1) {
        if (v >= s3) V[v].newid = (i32)k3++;
        else if (v >= s2) V[v].newid = (i32)k2++;
        else V[v].newid = (i32)k1++;
      }
    }
  }
  for (i64 i = 0; i < n; ++i) {
    if (V[i].newid == -1) {
      if (i >= s3) V[i].newid = (i32)k3++;
      else if (i >= s2) V[i].newid = (i32)k2++;
      else V[i].newid = (i32)k1++;
    }
  }
  /* rows in new-id order, neighbour order kept */
  i64 *len = (i64 *)calloc((size_t)(n + 1), sizeof(i64));
  for (i64 i = 0; i < n; ++i) len[V[i].newid] = V[i].len;
  beg[0] = 0;
  for (i64 i = 0; i < n; ++i) beg[i + 1] = beg[i] + len[i];
  for (i64 i = 0; i < n; ++i) {
    i64 o = beg[V[i].newid];
    for (i64 j = 0; j < V[i].len; ++j) adj[o + j] = V[V[i].e[j]].newid;
  }
  if (s2_out) *s2_out = s2;
  if (s3_out) *s3_out = s3;
  for (i64 i = 0; i < n; ++i) free(V[i].e);
  free(V); free(a); free(len);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* partition (Preprocess/partition.cpp:72-121)                                                 */
/* ------------------------------------------------------------------------------------------ */
/* Tile (i,j): rows = vertices v with v%p == i (local row v/p), values w/p for w%p == j.
 * tile_beg[(i*p+j)] must hold rows_i+1 int64, tile_adj[(i*p+j)] the tile's entries. */
int orc_partition_sizes(const i64 *beg, const i32 *adj, i64 n, int p, i64 *rows, i64 *ents) {
  for (int i = 0; i < p; ++i) rows[i] = (n - i + p - 1) / p;
  for (int t = 0; t < p * p; ++t) ents[t] = 0;
  for (i64 v = 0; v < n; ++v)
    for (i64 k = beg[v]; k < beg[v + 1]; ++k) ents[(v % p) * p + adj[k] % p]++;
  return 0;
}

int orc_partition(const i64 *beg, const i32 *adj, i64 n, int p, i64 **tile_beg, i32 **tile_adj) {
  i64 *fill = (i64 *)calloc((size_t)p * p, sizeof(i64));
  for (int t = 0; t < p * p; ++t) tile_beg[t][0] = 0;
  for (i64 v = 0; v < n; ++v) {
    int ii = (int)(v % p);
    i64 r = v / p;
    for (i64 k = beg[v]; k < beg[v + 1]; ++k) {
      int jj = adj[k] % p;
      tile_adj[ii * p + jj][fill[ii * p + jj]++] = adj[k] / p;
    }
    for (int j = 0; j < p; ++j) tile_beg[ii * p + j][r + 1] = fill[ii * p + j];
  }
  free(fill);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* counter-based generators (CPU twins of the product's GPU generators)                        */
/* ------------------------------------------------------------------------------------------ */
static inline u64 mix64(u64 x) { /* splitmix64 finaliser (Steele, Lea, Flood 2014) */
  x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
  x ^= x >> 27; x *= 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}
static inline u64 draw(u64 key, u64 i, u64 j) { return mix64(key + (i * 64 + j) * 0x9E3779B97F4A7C15ULL); }
u64 orc_gen_key(u64 seed) { return mix64(seed ^ 0x243F6A8885A308D3ULL); }

/* R-MAT: thresholds are cumulative quadrant probabilities scaled by 2^32 (ta < tab < tabc). */
void orc_gen_rmat(int scale, i64 np, uint32_t ta, uint32_t tab, uint32_t tabc, u64 seed, i32 *out) {
  u64 key = orc_gen_key(seed);
  for (i64 i = 0; i < np; ++i) {
    uint32_t u = 0, v = 0;
    for (int l = 0; l < scale; ++l) {
      uint32_t r = (uint32_t)(draw(key, (u64)i, (u64)l) >> 32);
      uint32_t ub = r >= tab, vb = (r >= ta && r < tab) || r >= tabc;
      u = (u << 1) | ub;
      v = (v << 1) | vb;
    }
    out[2 * i] = (i32)u;
    out[2 * i + 1] = (i32)v;
  }
}

/* Endpoint sampler over a cumulative table cdf[0..n-1] (non-decreasing, cdf[n-1] = 2^63). */
static i32 sample_cdf(const u64 *cdf, i64 n, u64 r) {
  i64 lo = 0, hi = n - 1;
  while (lo < hi) {
    i64 mid = (lo + hi) / 2;
    if (cdf[mid] > r) hi = mid; else lo = mid + 1;
  }
  return (i32)lo;
}

void orc_gen_weighted(const u64 *cdf, i64 n, i64 np, u64 seed, i32 *out) {
  u64 key = orc_gen_key(seed);
  for (i64 i = 0; i < np; ++i) {
    out[2 * i] = sample_cdf(cdf, n, draw(key, (u64)i, 0) >> 1);
    out[2 * i + 1] = sample_cdf(cdf, n, draw(key, (u64)i, 1) >> 1);
  }
}

void orc_gen_er(i64 n, i64 np, u64 seed, i32 *out) {
  u64 key = orc_gen_key(seed);
  for (i64 i = 0; i < np; ++i) {
    out[2 * i] = (i32)(((draw(key, (u64)i, 0) >> 32) * (u64)n) >> 32);
    out[2 * i + 1] = (i32)(((draw(key, (u64)i, 1) >> 32) * (u64)n) >> 32);
  }
}

/* Barabasi-Albert graph with d edges per vertex: n*d pairs (v, target), vertex 0's d pairs are
 * self loops.  The endpoint-copy method of Batagelj & Brandes (2005) in its per-edge form
 * (Sanders & Schulz 2016): edge e of vertex v = e/d >= 1 draws r uniformly in [0, 2 v d); an
 * even r names the source (r/2)/d, an odd r the target of edge (r-1)/2, resolved the same way.
 * Restated here so the generator in trust_gb300/csrc/tc_gen.cu can be checked bit for bit. */
static u64 ba_target(u64 key, u64 e, u64 d) {
  for (;;) {
    u64 v = e / d;
    if (v == 0) return 0;
    u64 r = (u64)(((unsigned __int128)draw(key, e, 0) * (2 * v * d)) >> 64);
    if ((r & 1) == 0) return (r >> 1) / d;
    e = r >> 1;
  }
}

void orc_gen_ba(i64 n, int d, u64 seed, i32 *out) {
  u64 key = orc_gen_key(seed);
  for (i64 e = 0; e < n * (i64)d; ++e) {
    out[2 * e] = (i32)(e / d);
    out[2 * e + 1] = (i32)ba_target(key, (u64)e, (u64)d);
  }
}

/* Chung-Lu expected degrees w_i = w_max * (1 + i/i0)^(-1/(gamma-1)), i0 chosen by bisection so
 * that the integral approximation of sum w equals 2*target_edges; cdf[i] = floor(2^63 * prefix_i /
 * total), cdf[n-1] = 2^63.  Returns i0. */
double orc_chung_lu_cdf(i64 n, double gamma, double w_max, i64 target_edges, u64 *cdf) {
  double alpha = 1.0 / (gamma - 1.0);
  double want = 2.0 * (double)target_edges;
  double lo = log(1e-3), hi = log(1e12);
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi), i0 = exp(mid), s;
    if (fabs(alpha - 1.0) < 1e-12) s = w_max * i0 * log(1.0 + (double)n / i0);
    else s = w_max * i0 / (1.0 - alpha) * (pow(1.0 + (double)n / i0, 1.0 - alpha) - 1.0);
    if (s < want) lo = mid; else hi = mid;
  }
  double i0 = exp(0.5 * (lo + hi));
  double total = 0.0;
  for (i64 i = 0; i < n; ++i) total += w_max * pow(1.0 + (double)i / i0, -alpha);
  double run = 0.0;
  for (i64 i = 0; i < n; ++i) {
    run += w_max * pow(1.0 + (double)i / i0, -alpha);
    double f = run / total;
    if (f > 1.0) f = 1.0;
    cdf[i] = (u64)(f * 9223372036854775808.0);
  }
  if (n > 0) cdf[n - 1] = (u64)1 << 63;
  return i0;
}
