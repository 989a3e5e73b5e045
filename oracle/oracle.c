/*
 * CPU oracle for the octree build: a plain-C restatement of the reference's
 * CPU stage functions (ucsc-redwood/pipeline, kernels/*.cpp and
 * include/shared/*.h), with OpenMP where the reference uses it.
 *
 * TEST INFRASTRUCTURE ONLY. The parity tests, smoke() and bench.py's CPU
 * baseline call it as the checker / the timed CPU reference; the product
 * (pipeline_gb300) never links, loads or calls it.
 *
 * Parity is pinned: tests/golden/ holds fixtures made by running the
 * reference's own sources (oracle/build_ref.sh + tests/golden/make_golden.py),
 * and tests/test_oracle_golden.py checks this file against them.
 *
 * Contract conventions where the reference drivers leave behaviour undefined
 * (each one is applied identically by the CUDA path):
 *   O1  the radix tree gets n = U-1 (apps/cpu_demo/main.cpp:95,102);
 *   O2  edge count / prefix sum run over B = U-1 entries;
 *   O3  number of octree nodes M = (largest slot any write touches) + 1, which
 *       equals prefix_sum[B-1] + 1 whenever the reference stays in bounds;
 *   O4  every output buffer starts zeroed (OctNodes, parent[]);
 *   O6  stages 7-8 are sequential in ascending i (1 thread), LinkLeaf's left
 *       write before its right write;
 *   O7  the LinkLeaf walk stops at radix node 0 (the reference loops forever
 *       there, include/shared/oct.h:111-113);
 *   O8  FP32 with no contraction (compile with -ffp-contract=off);
 *   O10 a shift by a negative count (leaf level 11, oct.h:106-107) shifts by
 *       the count modulo 32, as x86-64 and aarch64 shifters do;
 *   O11 a one-node tree (U = 2) takes clz(0) = 32 and skips the out-of-range
 *       parent write (kernels/04_radix_tree.cpp:117-118 would write parent[1]).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MORTON_BITS 30

typedef struct {
  int32_t children[8];
  float corner[4];
  float cell_size;
  int32_t child_node_mask;
  int32_t child_leaf_mask;
} orc_octnode;

_Static_assert(sizeof(orc_octnode) == 60, "OctNode layout is 60 bytes");

static int g_threads = 1;

void orc_set_threads(int n) {
  g_threads = n < 1 ? 1 : n;
#ifdef _OPENMP
  omp_set_num_threads(g_threads);
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Stage 0: input generator. kernels/00_init.cpp:20-30 draws                 */
/* glm::vec4(dis(gen), dis(gen), dis(gen), 1) from std::mt19937(seed) and     */
/* std::uniform_real_distribution<float>(min, min + range). Restated from the */
/* published MT19937 algorithm and the C++ generate_canonical<float, 24>      */
/* rule (one 32-bit draw, u / 2^32 in float, clamped below 1), as libstdc++   */
/* (GCC 13) implements them. GCC evaluates the three constructor arguments    */
/* right to left, so the first draw becomes z and the third x.                */
/* ------------------------------------------------------------------------ */
typedef struct {
  uint32_t mt[624];
  int idx;
} orc_mt19937;

static void mt_seed(orc_mt19937* s, uint32_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < 624; ++i)
    s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
  s->idx = 624;
}

static uint32_t mt_next(orc_mt19937* s) {
  if (s->idx >= 624) {
    for (int i = 0; i < 624; ++i) {
      uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
      uint32_t v = s->mt[(i + 397) % 624] ^ (y >> 1);
      if (y & 1u) v ^= 0x9908b0dfu;
      s->mt[i] = v;
    }
    s->idx = 0;
  }
  uint32_t y = s->mt[s->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

static float canonical_float(orc_mt19937* s) {
  float r = (float)mt_next(s) / 4294967296.0f;
  if (r >= 1.0f) r = nextafterf(1.0f, 0.0f);
  return r;
}

void orc_init_random_vec4(float* out, int n, float min, float range, int seed) {
  orc_mt19937 s;
  mt_seed(&s, (uint32_t)seed);
  const float hi = min + range;
  const float span = hi - min;
  for (int i = 0; i < n; ++i) {
    float a = canonical_float(&s) * span + min;
    float b = canonical_float(&s) * span + min;
    float c = canonical_float(&s) * span + min;
    out[4 * (size_t)i + 0] = c;
    out[4 * (size_t)i + 1] = b;
    out[4 * (size_t)i + 2] = a;
    out[4 * (size_t)i + 3] = 1.0f;
  }
}

/* The reference's device generator (kernels/cuda/00_init.cu:11-50) as its   */
/* driver launches it (apps/gpu_demo/main.cu:168-175: ceil(n/768) blocks of   */
/* 768 threads, so thread i makes element i): four 32-bit states seeded with  */
/* (4i + k) * seed, one step of the hybrid Tausworthe/LCG generator (three    */
/* Tausworthe steps + an LCG, GPU Gems 3 ch. 37), and the low 24 bits of      */
/* z1^z2, z2^z3, z3^z4, z1^z4 mapped to min + u / 2^24 * range. nvcc's default */
/* contraction makes that last step one fused multiply-add, so fmaf here.      */
void orc_init_random_vec4_gpu(float* out, int n, float min, float range, int seed) {
  const uint32_t sd = (uint32_t)seed;
  for (int i = 0; i < n; ++i) {
    const uint32_t b = (uint32_t)i << 2;
    uint32_t z1 = b * sd, z2 = (b + 1u) * sd, z3 = (b + 2u) * sd, z4 = (b + 3u) * sd;
    z1 = ((z1 & 4294967294u) << 12) ^ (((z1 << 13) ^ z1) >> 19);
    z2 = ((z2 & 4294967288u) << 4) ^ (((z2 << 2) ^ z2) >> 25);
    z3 = ((z3 & 4294967280u) << 17) ^ (((z3 << 3) ^ z3) >> 11);
    z4 = z4 * 1664525u + 1013904223u;
    const uint32_t v[4] = {z1 ^ z2, z2 ^ z3, z3 ^ z4, z1 ^ z4};
    for (int k = 0; k < 4; ++k)
      out[4 * (size_t)i + k] = fmaf((float)(v[k] & 0xFFFFFFu) / 16777216.0f, range, min);
  }
}

/* ------------------------------------------------------------------------ */
/* Stage 1: Morton encode (include/shared/morton.h:15-39,                     */
/* kernels/01_morton.cpp:5-14). Quantise each axis as (v - min) / range *     */
/* 1024 in FP32, in that order, truncate to uint32, keep 10 bits, interleave  */
/* x at bit 0, y at bit 1, z at bit 2.                                        */
/* ------------------------------------------------------------------------ */
static inline uint32_t spread3(uint32_t v) {
  uint32_t x = v & 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

static inline uint32_t compact3(uint32_t m) {
  uint32_t x = m & 0x09249249u;
  x = (x ^ (x >> 2)) & 0x030c30c3u;
  x = (x ^ (x >> 4)) & 0x0300f00fu;
  x = (x ^ (x >> 8)) & 0x030000ffu;
  x = (x ^ (x >> 16)) & 0x000003ffu;
  return x;
}

static inline uint32_t quantise(float v, float min, float range) {
  float q = (v - min) / range * 1024.0f;
  return (uint32_t)q;
}

void orc_morton(const float* pts, uint32_t* keys, long n, float min, float range) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    const float* p = pts + 4 * (size_t)i;
    keys[i] = spread3(quantise(p[0], min, range)) | (spread3(quantise(p[1], min, range)) << 1) |
              (spread3(quantise(p[2], min, range)) << 2);
  }
}

/* morton.h:60-80: corner = (raw / 1024) * range + min per axis, w = 1. */
static void decode_corner(float* out, uint32_t code, float min, float range) {
  for (int a = 0; a < 3; ++a) {
    float raw = (float)compact3(code >> a);
    float t = raw / 1024.0f;
    t = t * range;
    out[a] = t + min;
  }
  out[3] = 1.0f;
}

/* morton32_to_xyz over an array (include/shared/morton.h:45-80). */
void orc_morton_decode(const uint32_t* codes, long n, float min, float range, float* out) {
  for (long i = 0; i < n; ++i) decode_corner(out + 4 * (size_t)i, codes[i], min, range);
}

/* checkTree (apps/cpu_demo/main.cpp:13-35) without recursion: from node      */
/* oct_idx with (prefix, code_len), every child_node_mask bit continues at    */
/* children[c] with (prefix << 3 | c, code_len + 3); every child_leaf_mask   */
/* bit compares codes[children[c]] >> (30 - (code_len + 3)) with the child's  */
/* prefix. Counts {nodes visited, leaf checks, mismatches, rejected}: a       */
/* rejected step is a child index outside the arrays or a depth past 30 bits  */
/* (where the reference would shift by a negative count or recurse forever).  */
typedef struct {
  int node;
  uint32_t prefix;
  int len;
} orc_visit;

void orc_check_tree(const orc_octnode* nodes, int n_nodes, const uint32_t* codes, int n_codes,
                    uint32_t prefix, int code_len, int oct_idx, long long* counts) {
  counts[0] = counts[1] = counts[2] = counts[3] = 0;
  if (oct_idx < 0 || oct_idx >= n_nodes) {
    counts[3] = 1;
    return;
  }
  size_t cap = 1024, top = 0;
  orc_visit* stack = (orc_visit*)malloc(cap * sizeof(orc_visit));
  stack[top++] = (orc_visit){oct_idx, prefix, code_len};
  while (top > 0) {
    const orc_visit v = stack[--top];
    const orc_octnode* nd = &nodes[v.node];
    counts[0]++;
    for (int c = 0; c < 8; ++c) {
      const uint32_t np = (v.prefix << 3) | (uint32_t)c;
      if (nd->child_node_mask & (1 << c)) {
        const int q = nd->children[c];
        if (q < 0 || q >= n_nodes || v.len + 3 > MORTON_BITS) {
          counts[3]++;
        } else {
          if (top == cap) {
            cap *= 2;
            stack = (orc_visit*)realloc(stack, cap * sizeof(orc_visit));
          }
          stack[top++] = (orc_visit){q, np, v.len + 3};
        }
      }
      if (nd->child_leaf_mask & (1 << c)) {
        const int leaf = nd->children[c];
        if (leaf < 0 || leaf >= n_codes || v.len + 3 > MORTON_BITS) {
          counts[3]++;
        } else {
          counts[1]++;
          if ((codes[leaf] >> (MORTON_BITS - (v.len + 3))) != np) counts[2]++;
        }
      }
    }
  }
  free(stack);
}

/* ------------------------------------------------------------------------ */
/* Stage 2: sort (kernels/02_sort.cpp:13-58). Keys-only LSD radix sort with   */
/* 8-bit digits and four passes; each thread histograms its static block,     */
/* offsets are assigned thread by thread, and the scatter is stable.          */
/* ------------------------------------------------------------------------ */
void orc_radix_sort(uint32_t* keys, int n) {
  if (n <= 1) return;
  uint32_t* buf = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
  uint32_t* src = keys;
  uint32_t* dst = buf;
  int nt = g_threads;
  int(*hist)[256] = (int(*)[256])calloc((size_t)nt, sizeof(int[256]));
  for (int shift = 0; shift < 32; shift += 8) {
    memset(hist, 0, (size_t)nt * sizeof(int[256]));
#pragma omp parallel num_threads(nt)
    {
      int t = 0, T = 1;
#ifdef _OPENMP
      t = omp_get_thread_num();
      T = omp_get_num_threads();
#endif
      long lo = (long)n * t / T, hi = (long)n * (t + 1) / T;
      for (long i = lo; i < hi; ++i) hist[t][(src[i] >> shift) & 0xffu]++;
#pragma omp barrier
#pragma omp single
      {
        int run = 0;
        for (int d = 0; d < 256; ++d)
          for (int u = 0; u < T; ++u) {
            int c = hist[u][d];
            hist[u][d] = run;
            run += c;
          }
      }
      for (long i = lo; i < hi; ++i) dst[hist[t][(src[i] >> shift) & 0xffu]++] = src[i];
    }
    uint32_t* tmp = src;
    src = dst;
    dst = tmp;
  }
  /* four passes: the result is back in keys */
  free(hist);
  free(buf);
}

/* ------------------------------------------------------------------------ */
/* Stage 3: unique (kernels/03_unique.cpp:2-16). In-place compaction of runs  */
/* of equal keys; returns U; entries [U, n) keep their old values.            */
/* ------------------------------------------------------------------------ */
int orc_count_unique(uint32_t* keys, int n) {
  if (n == 0) return 0;
  int j = 0;
  for (int i = 1; i < n; ++i)
    if (keys[i] != keys[j]) keys[++j] = keys[i];
  return j + 1;
}

/* ------------------------------------------------------------------------ */
/* Stage 4: Karras radix tree (kernels/04_radix_tree.cpp:16-121). Node i in   */
/* [0, n) over the n+1 keys codes[0..n]. The search steps are the            */
/* reference's, kept step for step because every quirk shows in the output: */
/* the root takes d = 1 and l = n - 1 (so it spans keys [0, n-1]); the       */
/* exponential search doubles l_max from 2 while i + l_max*d stays in        */
/* [0, n]; the binary searches honour l_cutoff and s_cutoff.                 */
/* ------------------------------------------------------------------------ */
static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }
/* delta_u32 returns uint8_t (04_radix_tree.cpp:21-27): clz - 1 wraps to 255
 * for keys that differ in bit 31. */
static inline int delta32(uint32_t a, uint32_t b) { return (uint8_t)(clz32(a ^ b) - 1); }
static inline int log2_ceil32(uint32_t x) {
  /* x >= 1 here */
  int fl = 31 - clz32(x);
  return fl + ((1u << fl) < x);
}

static void radix_node(int i, int n, const uint32_t* codes, uint8_t* prefix_n, uint8_t* hll,
                       uint8_t* hlr, int* left_child, int* parent) {
  const uint32_t ci = codes[i];
  int d;
  if (i == 0) {
    d = 1;
  } else {
    int diff = delta32(ci, codes[i + 1]) - delta32(ci, codes[i - 1]);
    d = (diff > 0) - (diff < 0);
  }
  int l = 0;
  if (i == 0) {
    l = n - 1;
  } else {
    const int dmin = delta32(ci, codes[i - d]);
    long lmax = 2;
    while (i + lmax * d >= 0 && i + lmax * d <= n && delta32(ci, codes[i + lmax * d]) > dmin)
      lmax *= 2;
    const int lcut = (d == -1) ? i : n - i;
    for (long t = lmax / 2, div = 2; t >= 1; div *= 2, t = lmax / div)
      if (l + t <= lcut && delta32(ci, codes[i + (l + t) * d]) > dmin) l += (int)t;
  }
  const int j = i + l * d;
  const int dnode = delta32(codes[i], codes[j]);
  prefix_n[i] = (uint8_t)dnode;
  int s = 0;
  if (l > 0) {
    const long maxdiv = 1L << log2_ceil32((uint32_t)l);
    const int scut = (d == -1) ? i - 1 : n - i - 1;
    long div = 2;
    for (long t = ((long)l + 1) / 2; div <= maxdiv; div <<= 1, t = ((long)l + div - 1) / div)
      if (s + t <= scut && delta32(ci, codes[i + (s + t) * d]) > dnode) s += (int)t;
  }
  const int gamma = i + s * d + (d < 0 ? d : 0);
  left_child[i] = gamma;
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  hll[i] = (uint8_t)(lo == gamma);
  hlr[i] = (uint8_t)(hi == gamma + 1);
  if (!hll[i] && gamma < n) parent[gamma] = i;
  if (!hlr[i] && gamma + 1 < n) parent[gamma + 1] = i;
}

/* Sequential (ascending i) so that, where two nodes write the same parent[]
 * entry, the later node's value stays, as a 1-thread run of the reference. */
void orc_build_radix_tree(int n, const uint32_t* codes, uint8_t* prefix_n, uint8_t* hll,
                          uint8_t* hlr, int* left_child, int* parent) {
  for (int i = 0; i < n; ++i) radix_node(i, n, codes, prefix_n, hll, hlr, left_child, parent);
}

/* Timing variant: the reference's `omp parallel for` over nodes. */
void orc_build_radix_tree_par(int n, const uint32_t* codes, uint8_t* prefix_n, uint8_t* hll,
                              uint8_t* hlr, int* left_child, int* parent) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) radix_node(i, n, codes, prefix_n, hll, hlr, left_child, parent);
}

/* ------------------------------------------------------------------------ */
/* Stage 5: edge count (kernels/05_edge_count.cpp:3-16).                      */
/* ------------------------------------------------------------------------ */
void orc_edge_count(const uint8_t* prefix_n, const int* parent, int* ec, int n) {
  if (n <= 0) return;
  ec[0] = 0;
#pragma omp parallel for schedule(static)
  for (int i = 1; i < n; ++i) ec[i] = prefix_n[i] / 3 - prefix_n[parent[i]] / 3;
}

/* ------------------------------------------------------------------------ */
/* Stage 6: inclusive prefix sum (kernels/06_partial_sum.cpp:3-15).           */
/* ------------------------------------------------------------------------ */
void orc_partial_sum(const int* data, long first, long last, int* out) {
  int sum = 0;
  for (long i = first; i < last; ++i) {
    sum += data[i];
    out[i - first] = sum;
  }
}

/* O3: one past the largest slot that stages 7-8 write. */
int orc_oct_node_count(const int* ec, const int* ps, int n) {
  if (n <= 0) return 0;
  long m = ps[n - 1];
  for (int i = 1; i < n; ++i)
    if (ec[i] > 0 && (long)ps[i] + ec[i] - 1 > m) m = (long)ps[i] + ec[i] - 1;
  return (int)(m + 1);
}

/* ------------------------------------------------------------------------ */
/* Stage 7: octree nodes (include/shared/oct.h:9-14, 24-90;                   */
/* kernels/07_octree.cpp:5-31) and the caller's root set-up                   */
/* (apps/cpu_demo/main.cpp:125-132).                                          */
/* ------------------------------------------------------------------------ */
void orc_root_init(orc_octnode* nodes, const uint32_t* codes, const uint8_t* prefix_n, float min,
                   float range) {
  const int root_level = prefix_n[0] / 3;
  const int sh = MORTON_BITS - 3 * root_level;
  decode_corner(nodes[0].corner, (codes[0] >> sh) << sh, min, range);
  nodes[0].cell_size = range;
}

static void oct_node(int i, orc_octnode* nodes, const int* offsets, const int* counts,
                     const uint32_t* codes, const uint8_t* prefix_n, const int* parents, float min,
                     float range) {
  int oct_idx = offsets[i];
  const int k = counts[i];
  const int root_level = prefix_n[0] / 3;
  for (int j = 0; j < k - 1; ++j) {
    const int level = prefix_n[i] / 3 - j;
    const int sh = MORTON_BITS - 3 * level;
    const uint32_t pre = codes[i] >> sh;
    const int which = (int)(pre & 7u);
    const int up = oct_idx + 1;
    nodes[up].children[which] = oct_idx;
    nodes[up].child_node_mask |= 1 << which;
    decode_corner(nodes[oct_idx].corner, pre << sh, min, range);
    nodes[oct_idx].cell_size = range / (float)(1 << (level - root_level));
    oct_idx = up;
  }
  if (k > 0) {
    int rp = parents[i];
    int counter = 0;
    while (counts[rp] == 0) {
      rp = parents[rp];
      if (++counter > 30) break;
    }
    const int oct_parent = offsets[rp];
    const int top = prefix_n[i] / 3 - k + 1;
    const int sh = MORTON_BITS - 3 * top;
    const uint32_t pre = codes[i] >> sh;
    const int which = (int)(pre & 7u);
    nodes[oct_parent].children[which] = oct_idx;
    nodes[oct_parent].child_node_mask |= 1 << which;
    decode_corner(nodes[oct_idx].corner, pre << sh, min, range);
    nodes[oct_idx].cell_size = range / (float)(1 << (top - root_level));
  }
}

void orc_make_oct_nodes(orc_octnode* nodes, const int* offsets, const int* counts,
                        const uint32_t* codes, const uint8_t* prefix_n, const int* parents,
                        float min, float range, int n) {
  for (int i = 1; i < n; ++i)
    oct_node(i, nodes, offsets, counts, codes, prefix_n, parents, min, range);
}

/* Timing variant: the reference's `omp parallel for` (racy, as there). */
void orc_make_oct_nodes_par(orc_octnode* nodes, const int* offsets, const int* counts,
                            const uint32_t* codes, const uint8_t* prefix_n, const int* parents,
                            float min, float range, int n) {
#pragma omp parallel for schedule(static)
  for (int i = 1; i < n; ++i)
    oct_node(i, nodes, offsets, counts, codes, prefix_n, parents, min, range);
}

/* ------------------------------------------------------------------------ */
/* Stage 8: leaf links (include/shared/oct.h:16-21, 92-134;                   */
/* kernels/07_octree.cpp:33-57). SetLeaf clears the leaf-mask bit, so on      */
/* zeroed nodes child_leaf_mask stays 0.                                      */
/* ------------------------------------------------------------------------ */
static void link_one(orc_octnode* nodes, const int* offsets, const int* counts,
                     const uint32_t* codes, const uint8_t* prefix_n, const int* parents, int i,
                     int leaf) {
  const int leaf_level = prefix_n[i] / 3 + 1;
  const uint32_t sh = (uint32_t)(MORTON_BITS - 3 * leaf_level) & 31u; /* O10 */
  const int which = (int)((codes[leaf] >> sh) & 7u);
  int r = i;
  while (counts[r] == 0 && r != 0) r = parents[r]; /* O7 */
  orc_octnode* nd = &nodes[offsets[r]];
  nd->children[which] = leaf;
  nd->child_leaf_mask &= ~(1 << which);
}

static void leaf_node(int i, orc_octnode* nodes, const int* offsets, const int* counts,
                      const uint32_t* codes, const uint8_t* hll, const uint8_t* hlr,
                      const uint8_t* prefix_n, const int* parents, const int* left_child) {
  if (hll[i]) link_one(nodes, offsets, counts, codes, prefix_n, parents, i, left_child[i]);
  if (hlr[i]) link_one(nodes, offsets, counts, codes, prefix_n, parents, i, left_child[i] + 1);
}

/* Number of LinkLeaf walks that reach radix node 0 with counts[0] == 0: the
 * inputs on which the reference's unbounded walk (oct.h:111-113) never ends
 * and contract O7 applies instead. Harness code checks this before it runs
 * the reference's own k_LinkLeafNodes. */
int orc_o7_walks(const int* counts, const uint8_t* hll, const uint8_t* hlr, const int* parents,
                 int n) {
  int hits = 0;
  for (int i = 0; i < n; ++i) {
    if (!hll[i] && !hlr[i]) continue;
    int r = i, steps = 0;
    while (counts[r] == 0 && r != 0 && steps++ < 64) r = parents[r];
    if (counts[r] == 0) hits += hll[i] + hlr[i];
  }
  return hits;
}

void orc_link_leaf_nodes(orc_octnode* nodes, const int* offsets, const int* counts,
                         const uint32_t* codes, const uint8_t* hll, const uint8_t* hlr,
                         const uint8_t* prefix_n, const int* parents, const int* left_child,
                         int n) {
  for (int i = 0; i < n; ++i)
    leaf_node(i, nodes, offsets, counts, codes, hll, hlr, prefix_n, parents, left_child);
}

void orc_link_leaf_nodes_par(orc_octnode* nodes, const int* offsets, const int* counts,
                             const uint32_t* codes, const uint8_t* hll, const uint8_t* hlr,
                             const uint8_t* prefix_n, const int* parents, const int* left_child,
                             int n) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i)
    leaf_node(i, nodes, offsets, counts, codes, hll, hlr, prefix_n, parents, left_child);
}

/* ------------------------------------------------------------------------ */
/* Whole build, in the order of apps/cpu_demo/main.cpp:72-154 with O1-O11.    */
/* Buffers (caller-owned, each n entries unless noted, nodes_cap OctNodes):   */
/* keys receives the Morton codes, then sorted, then unique in place.        */
/* When morton_out is non-NULL the unsorted codes are kept there.             */
/* stage_ms (8 doubles, optional) receives per-stage wall times.              */
/* Returns M, or -(needed M) if nodes_cap is too small.                       */
/* ------------------------------------------------------------------------ */
static double now_ms(void) {
#ifdef _OPENMP
  return omp_get_wtime() * 1e3;
#else
  return 0.0;
#endif
}

int orc_build_all(const float* pts, int n, float min, float range, int parallel_octree,
                  uint32_t* morton_out, uint32_t* keys, int* n_unique, uint8_t* prefix_n,
                  uint8_t* hll, uint8_t* hlr, int* left_child, int* parent, int* ec, int* ps,
                  orc_octnode* nodes, int nodes_cap, double* stage_ms) {
  double t[9];
  t[0] = now_ms();
  orc_morton(pts, keys, n, min, range);
  if (morton_out) memcpy(morton_out, keys, (size_t)n * sizeof(uint32_t));
  t[1] = now_ms();
  orc_radix_sort(keys, n);
  t[2] = now_ms();
  const int U = orc_count_unique(keys, n);
  *n_unique = U;
  t[3] = now_ms();
  const int B = U - 1;
  if (B < 1) {
    if (stage_ms)
      for (int s = 0; s < 8; ++s) stage_ms[s] = s < 3 ? t[s + 1] - t[s] : 0.0;
    return 0;
  }
  memset(parent, 0, (size_t)B * sizeof(int));
  if (parallel_octree)
    orc_build_radix_tree_par(B, keys, prefix_n, hll, hlr, left_child, parent);
  else
    orc_build_radix_tree(B, keys, prefix_n, hll, hlr, left_child, parent);
  t[4] = now_ms();
  orc_edge_count(prefix_n, parent, ec, B);
  t[5] = now_ms();
  orc_partial_sum(ec, 0, B, ps);
  ps[0] = 0;
  t[6] = now_ms();
  const int M = orc_oct_node_count(ec, ps, B);
  if (M > nodes_cap) return -M;
  memset(nodes, 0, (size_t)M * sizeof(orc_octnode));
  orc_root_init(nodes, keys, prefix_n, min, range);
  if (parallel_octree)
    orc_make_oct_nodes_par(nodes, ps, ec, keys, prefix_n, parent, min, range, B);
  else
    orc_make_oct_nodes(nodes, ps, ec, keys, prefix_n, parent, min, range, B);
  t[7] = now_ms();
  if (parallel_octree)
    orc_link_leaf_nodes_par(nodes, ps, ec, keys, hll, hlr, prefix_n, parent, left_child, B);
  else
    orc_link_leaf_nodes(nodes, ps, ec, keys, hll, hlr, prefix_n, parent, left_child, B);
  t[8] = now_ms();
  if (stage_ms)
    for (int s = 0; s < 8; ++s) stage_ms[s] = t[s + 1] - t[s];
  return M;
}

/* FNV-1a 64 over raw bytes: the fingerprint the golden fixtures record. */
uint64_t orc_fnv1a64(const void* data, size_t nbytes) {
  const unsigned char* p = (const unsigned char*)data;
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < nbytes; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}
