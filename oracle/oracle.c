/*
 * oracle.c -- CPU restatement of the reference's triangle BVH build and
 * stream ray queries.  TEST INFRASTRUCTURE ONLY: the checker for the GPU
 * library and the CPU baseline beside it; never linked into the product.
 * See oracle.h for the list of reference files:lines restated here and for
 * the two documented deviations.
 *
 * Compile with -ffp-contract=off: the reference's arithmetic fuses exactly
 * where it calls madd/msub (AVX2 build), which this file spells as fmaf();
 * every other operation must round on its own.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* common/math/constants.h:31-34 */
#define REF_FLT_LARGE 1.844E18f
#define REF_MIN_RCP_INPUT 1E-18f
#define INVALID_ID 0xFFFFFFFFu

/* builder settings: kernels/bvh/bvh_builder_sah.cpp:565 + bvh.h:71-73 +
   bvh_builder_sah.h:28 */
#define BINS 32
#define BRANCHING 8
#define LOG_BLOCK 2
#define MIN_LEAF 4
#define MAX_LEAF 28 /* 7 Triangle4 blocks (bvh_node_ref.h:92) */
#define MAX_DEPTH 40
#define MIN_LARGE_LEAF_LEVELS 8

#define EMPTY_REF 0xFFFFFFFFu
#define LEAF_BIT 0x80000000u

typedef struct { float x, y, z; } v3;

static inline v3 v3sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 v3mul(v3 a, v3 b) { v3 r = {a.x * b.x, a.y * b.y, a.z * b.z}; return r; }
/* dot(a,b) = madd(a.x,b.x,madd(a.y,b.y,a.z*b.z))   common/math/vec3.h:204 */
static inline float dot3(v3 a, v3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
/* cross via prod_diff(a,b,c,d) = msub(a,b,c*d)  vec3.h:209, math.h:367-373 */
static inline v3 cross3(v3 a, v3 b) {
  v3 r = {fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x))};
  return r;
}
static inline float fmin2(float a, float b) { return a < b ? a : b; }
static inline float fmax2(float a, float b) { return a > b ? a : b; }
static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* ------------------------------------------------------------------------ */
/* scene storage                                                            */
/* ------------------------------------------------------------------------ */

typedef struct {
  unsigned geomID;
  float* v;       /* 3*nv */
  unsigned nv;
  unsigned* idx;  /* 3*nt */
  unsigned nt;
} OMesh;

typedef struct {
  float lo[3], hi[3];
  unsigned geomID, primID;
} OPrim;

/* Triangle4: v0, e1 = v0-v1, e2 = v2-v0, ids; unused lanes geomID = -1
   (kernels/geometry/triangle.h:13-41, 98-120) */
typedef struct {
  float v0[3][4], e1[3][4], e2[3][4];
  unsigned geomID[4], primID[4];
} OTri4;

/* 8-wide node with SoA child boxes (kernels/bvh/bvh_node_aabb.h:200-205);
   empty slots carry (+inf,-inf) boxes (bvh_node_aabb.h:82-85). */
typedef struct {
  float lo[3][8], hi[3][8];
  uint32_t child[8];
} ONode8;

typedef struct { uint32_t first, nblocks; } OLeaf;

struct OracleScene {
  OMesh* meshes;
  size_t nmeshes, capmeshes;
  OPrim* prims;
  size_t nprims;
  ONode8* nodes;
  size_t nnodes, capnodes;
  OLeaf* leaves;
  size_t nleaves, capleaves;
  OTri4* tris;
  size_t ntris4, captris4;
  uint32_t root;
  float glo[3], ghi[3];
  int committed;
  int robust; /* RTC_SCENE_FLAG_ROBUST: Triangle4v leaves + Pluecker test */
  orc_filter_fn ifilter, ofilter; /* filter callbacks (NULL: none) and their argument */
  void* filter_user;
  pthread_mutex_t lock;
};

void orc_scene_set_filters(OracleScene* s, orc_filter_fn ifilter, orc_filter_fn ofilter, void* user) {
  s->ifilter = ifilter;
  s->ofilter = ofilter;
  s->filter_user = user;
}

OracleScene* orc_scene_new(void) {
  OracleScene* s = (OracleScene*)calloc(1, sizeof(OracleScene));
  s->root = EMPTY_REF;
  pthread_mutex_init(&s->lock, NULL);
  return s;
}

static void free_build(OracleScene* s) {
  free(s->prims); s->prims = NULL; s->nprims = 0;
  free(s->nodes); s->nodes = NULL; s->nnodes = s->capnodes = 0;
  free(s->leaves); s->leaves = NULL; s->nleaves = s->capleaves = 0;
  free(s->tris); s->tris = NULL; s->ntris4 = s->captris4 = 0;
  s->root = EMPTY_REF;
}

void orc_scene_free(OracleScene* s) {
  if (!s) return;
  for (size_t i = 0; i < s->nmeshes; i++) { free(s->meshes[i].v); free(s->meshes[i].idx); }
  free(s->meshes);
  free_build(s);
  pthread_mutex_destroy(&s->lock);
  free(s);
}

int orc_scene_add_mesh(OracleScene* s, unsigned geomID, const void* verts, size_t vstride, unsigned nverts,
                       const void* idx, size_t istride, unsigned ntris) {
  if (s->nmeshes == s->capmeshes) {
    s->capmeshes = s->capmeshes ? 2 * s->capmeshes : 8;
    s->meshes = (OMesh*)realloc(s->meshes, s->capmeshes * sizeof(OMesh));
  }
  OMesh* m = &s->meshes[s->nmeshes++];
  m->geomID = geomID;
  m->nv = nverts;
  m->nt = ntris;
  m->v = (float*)malloc((size_t)3 * nverts * sizeof(float) + 16);
  m->idx = (unsigned*)malloc((size_t)3 * ntris * sizeof(unsigned) + 16);
  for (unsigned i = 0; i < nverts; i++) memcpy(&m->v[3 * (size_t)i], (const char*)verts + i * vstride, 12);
  for (unsigned i = 0; i < ntris; i++) memcpy(&m->idx[3 * (size_t)i], (const char*)idx + i * istride, 12);
  s->committed = 0;
  return 0;
}

void orc_scene_set_robust(OracleScene* s, int robust) {
  s->robust = robust;
  s->committed = 0;
}

static int cmp_mesh(const void* a, const void* b) {
  unsigned ga = ((const OMesh*)a)->geomID, gb = ((const OMesh*)b)->geomID;
  return ga < gb ? -1 : ga > gb;
}

static const OMesh* find_mesh(const OracleScene* s, unsigned geomID) {
  size_t lo = 0, hi = s->nmeshes;
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if (s->meshes[mid].geomID < geomID) lo = mid + 1; else hi = mid;
  }
  if (lo < s->nmeshes && s->meshes[lo].geomID == geomID) return &s->meshes[lo];
  return NULL;
}

static inline v3 mesh_vertex(const OMesh* m, unsigned i) {
  v3 r = {m->v[3 * (size_t)i], m->v[3 * (size_t)i + 1], m->v[3 * (size_t)i + 2]};
  return r;
}

/* isvalid(Vec3fa): all(v > -FLT_LARGE & v < FLT_LARGE)  common/math/vec3fa.h:328 */
static inline int vertex_valid(v3 v) {
  return v.x > -REF_FLT_LARGE && v.x < REF_FLT_LARGE && v.y > -REF_FLT_LARGE && v.y < REF_FLT_LARGE &&
         v.z > -REF_FLT_LARGE && v.z < REF_FLT_LARGE;
}

/* ------------------------------------------------------------------------ */
/* builder                                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  size_t begin, end, depth;
  float glo[3], ghi[3]; /* geometry bounds */
  float clo[3], chi[3]; /* bounds of center2 = lower+upper */
} BRec;

typedef struct {
  float sah;
  int dim, pos;
  size_t num;
  float ofs[3], scale[3];
} BSplit;

/* halfArea(d) = madd(d.x,(d.y+d.z),d.y*d.z)  common/math/vec3fa.h:373 */
static inline float half_area3(const float lo[3], const float hi[3]) {
  float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  return fmaf(dx, dy + dz, dy * dz);
}

static inline void bb_empty(float lo[3], float hi[3]) {
  for (int d = 0; d < 3; d++) { lo[d] = INFINITY; hi[d] = -INFINITY; }
}
static inline void bb_extend(float lo[3], float hi[3], const float plo[3], const float phi[3]) {
  for (int d = 0; d < 3; d++) { lo[d] = fmin2(lo[d], plo[d]); hi[d] = fmax2(hi[d], phi[d]); }
}
static inline void center2(const OPrim* p, float c[3]) {
  for (int d = 0; d < 3; d++) c[d] = p->lo[d] + p->hi[d];
}

static void rec_init(BRec* r, const OPrim* prims, size_t b, size_t e, size_t depth) {
  r->begin = b; r->end = e; r->depth = depth;
  bb_empty(r->glo, r->ghi);
  bb_empty(r->clo, r->chi);
  for (size_t i = b; i < e; i++) {
    float c[3];
    center2(&prims[i], c);
    bb_extend(r->glo, r->ghi, prims[i].lo, prims[i].hi);
    bb_extend(r->clo, r->chi, c, c);
  }
}

/* BinMapping(N, centBounds)  kernels/builders/heuristic_binning.h:22-30 */
static void bin_mapping(BSplit* sp, const BRec* r) {
  size_t N = r->end - r->begin;
  size_t num = (size_t)(4.0f + 0.05f * (float)N);
  if (num > BINS) num = BINS;
  sp->num = num;
  const float eps = 1E-34f;
  for (int d = 0; d < 3; d++) {
    float diag = fmax2(eps, r->chi[d] - r->clo[d]);
    sp->scale[d] = diag > eps ? (0.99f * (float)num) / diag : 0.0f;
    sp->ofs[d] = r->clo[d];
  }
}

static inline int bin_of(const BSplit* sp, const float c[3], int d) {
  return (int)floorf((c[d] - sp->ofs[d]) * sp->scale[d]);
}

/* find(): binning + best()  heuristic_binning.h:211-260, 340-399 */
static BSplit find_split(const OPrim* prims, const BRec* r) {
  BSplit sp;
  bin_mapping(&sp, r);
  const size_t num = sp.num;
  float blo[BINS][3][3], bhi[BINS][3][3];
  unsigned cnt[BINS][3];
  for (size_t i = 0; i < num; i++)
    for (int d = 0; d < 3; d++) { bb_empty(blo[i][d], bhi[i][d]); cnt[i][d] = 0; }
  for (size_t i = r->begin; i < r->end; i++) {
    float c[3];
    center2(&prims[i], c);
    for (int d = 0; d < 3; d++) {
      int b = bin_of(&sp, c, d);
      if (b < 0) b = 0;
      if ((size_t)b >= num) b = (int)num - 1;
      bb_extend(blo[b][d], bhi[b][d], prims[i].lo, prims[i].hi);
      cnt[b][d] += 1;
    }
  }
  /* right-to-left sweep */
  float rArea[BINS][3];
  unsigned rCount[BINS][3];
  {
    unsigned count[3] = {0, 0, 0};
    float lo[3][3], hi[3][3];
    for (int d = 0; d < 3; d++) bb_empty(lo[d], hi[d]);
    for (size_t i = num - 1; i > 0; i--) {
      for (int d = 0; d < 3; d++) {
        count[d] += cnt[i][d];
        rCount[i][d] = count[d];
        bb_extend(lo[d], hi[d], blo[i][d], bhi[i][d]);
        rArea[i][d] = half_area3(lo[d], hi[d]);
      }
    }
  }
  /* left-to-right sweep */
  const unsigned blocks_add = (1u << LOG_BLOCK) - 1;
  float bestSAHd[3] = {INFINITY, INFINITY, INFINITY};
  unsigned bestPosd[3] = {0, 0, 0};
  {
    unsigned count[3] = {0, 0, 0};
    float lo[3][3], hi[3][3];
    for (int d = 0; d < 3; d++) bb_empty(lo[d], hi[d]);
    for (size_t i = 1; i < num; i++) {
      for (int d = 0; d < 3; d++) {
        count[d] += cnt[i - 1][d];
        bb_extend(lo[d], hi[d], blo[i - 1][d], bhi[i - 1][d]);
        float lA = half_area3(lo[d], hi[d]);
        unsigned lC = (count[d] + blocks_add) >> LOG_BLOCK;
        unsigned rC = (rCount[i][d] + blocks_add) >> LOG_BLOCK;
        float sah = fmaf(lA, (float)lC, rArea[i][d] * (float)rC);
        if (sah < bestSAHd[d]) { bestPosd[d] = (unsigned)i; bestSAHd[d] = sah; }
      }
    }
  }
  sp.sah = INFINITY;
  sp.dim = -1;
  sp.pos = 0;
  for (int d = 0; d < 3; d++) {
    if (sp.scale[d] == 0.0f) continue;
    if (bestSAHd[d] < sp.sah && bestPosd[d] != 0) {
      sp.dim = d;
      sp.pos = (int)bestPosd[d];
      sp.sah = bestSAHd[d];
    }
  }
  return sp;
}

static int cmp_prim_id(const void* a, const void* b) {
  const OPrim* pa = (const OPrim*)a;
  const OPrim* pb = (const OPrim*)b;
  uint64_t ia = ((uint64_t)pa->primID << 32) + pa->geomID;
  uint64_t ib = ((uint64_t)pb->primID << 32) + pb->geomID;
  return ia < ib ? -1 : ia > ib;
}

/* deterministic_order: heuristic_binning_array_aligned.h:123-127 */
static void deterministic_order(OPrim* prims, const BRec* r) {
  qsort(prims + r->begin, r->end - r->begin, sizeof(OPrim), cmp_prim_id);
}

/* splitFallback: middle split  heuristic_binning_array_aligned.h:129-144 */
static void split_fallback(const OPrim* prims, const BRec* r, BRec* l, BRec* rr) {
  size_t center = (r->begin + r->end) / 2;
  rec_init(l, prims, r->begin, center, r->depth + 1);
  rec_init(rr, prims, center, r->end, r->depth + 1);
}

typedef struct {
  OPrim* tmp;
} BuildCtx;

/* split(): partition by bin < pos along dim  heuristic_binning_array_aligned.h:78-121 */
static void do_split(OracleScene* s, BuildCtx* bc, const BSplit* sp, BRec* r, BRec* l, BRec* rr) {
  OPrim* prims = s->prims;
  if (sp->dim < 0) {
    deterministic_order(prims, r);
    split_fallback(prims, r, l, rr);
    return;
  }
  size_t nl = 0, nr = 0, n = r->end - r->begin;
  OPrim* tmp = bc->tmp;
  /* stable two-way partition: lefts in order, then rights in order */
  for (size_t i = r->begin; i < r->end; i++) {
    float c[3];
    center2(&prims[i], c);
    if (bin_of(sp, c, sp->dim) < sp->pos) prims[r->begin + nl++] = prims[i];
    else tmp[nr++] = prims[i];
  }
  memcpy(prims + r->begin + nl, tmp, nr * sizeof(OPrim));
  (void)n;
  rec_init(l, prims, r->begin, r->begin + nl, r->depth + 1);
  rec_init(rr, prims, r->begin + nl, r->end, r->depth + 1);
}

static uint32_t alloc_node(OracleScene* s) {
  if (s->nnodes == s->capnodes) {
    s->capnodes = s->capnodes ? 2 * s->capnodes : 1024;
    s->nodes = (ONode8*)realloc(s->nodes, s->capnodes * sizeof(ONode8));
  }
  ONode8* n = &s->nodes[s->nnodes];
  for (int i = 0; i < 8; i++) {
    for (int d = 0; d < 3; d++) { n->lo[d][i] = INFINITY; n->hi[d][i] = -INFINITY; }
    n->child[i] = EMPTY_REF;
  }
  return (uint32_t)s->nnodes++;
}

/* CreateLeaf -> Triangle4::fill  bvh_builder_sah.cpp:31-54, triangle.h:98-120 */
static uint32_t create_leaf(OracleScene* s, const BRec* r) {
  size_t n = r->end - r->begin;
  size_t blocks = (n + 3) / 4;
  if (s->ntris4 + blocks > s->captris4) {
    while (s->ntris4 + blocks > s->captris4) s->captris4 = s->captris4 ? 2 * s->captris4 : 1024;
    s->tris = (OTri4*)realloc(s->tris, s->captris4 * sizeof(OTri4));
  }
  if (s->nleaves == s->capleaves) {
    s->capleaves = s->capleaves ? 2 * s->capleaves : 1024;
    s->leaves = (OLeaf*)realloc(s->leaves, s->capleaves * sizeof(OLeaf));
  }
  uint32_t first = (uint32_t)s->ntris4;
  size_t k = r->begin;
  for (size_t b = 0; b < blocks; b++) {
    OTri4* t = &s->tris[s->ntris4++];
    for (int i = 0; i < 4; i++) {
      if (k < r->end) {
        const OPrim* p = &s->prims[k++];
        const OMesh* m = find_mesh(s, p->geomID);
        const unsigned* tri = &m->idx[3 * (size_t)p->primID];
        v3 p0 = mesh_vertex(m, tri[0]), p1 = mesh_vertex(m, tri[1]), p2 = mesh_vertex(m, tri[2]);
        /* Triangle4 keeps edges (triangle.h:40-41); Triangle4v of robust
           scenes keeps the vertices (trianglev.h:93-115) in the same slots */
        v3 e1 = s->robust ? p1 : v3sub(p0, p1), e2 = s->robust ? p2 : v3sub(p2, p0);
        t->v0[0][i] = p0.x; t->v0[1][i] = p0.y; t->v0[2][i] = p0.z;
        t->e1[0][i] = e1.x; t->e1[1][i] = e1.y; t->e1[2][i] = e1.z;
        t->e2[0][i] = e2.x; t->e2[1][i] = e2.y; t->e2[2][i] = e2.z;
        t->geomID[i] = p->geomID;
        t->primID[i] = p->primID;
      } else {
        for (int d = 0; d < 3; d++) { t->v0[d][i] = 0; t->e1[d][i] = 0; t->e2[d][i] = 0; }
        t->geomID[i] = INVALID_ID;
        t->primID[i] = INVALID_ID;
      }
    }
  }
  s->leaves[s->nleaves].first = first;
  s->leaves[s->nleaves].nblocks = (uint32_t)blocks;
  return LEAF_BIT | (uint32_t)s->nleaves++;
}

static void set_child(OracleScene* s, uint32_t node, int slot, const BRec* c, uint32_t ref) {
  ONode8* n = &s->nodes[node];
  for (int d = 0; d < 3; d++) { n->lo[d][slot] = c->glo[d]; n->hi[d][slot] = c->ghi[d]; }
  n->child[slot] = ref;
}

/* createLargeLeaf  bvh_builder_sah.h:155-220 */
static uint32_t create_large_leaf(OracleScene* s, BuildCtx* bc, const BRec* cur) {
  if (cur->depth > MAX_DEPTH) return EMPTY_REF; /* "depth limit reached" */
  if (cur->end - cur->begin <= MAX_LEAF) return create_leaf(s, cur);
  BRec children[BRANCHING];
  size_t n = 1;
  children[0] = *cur;
  do {
    int best = -1;
    size_t bestSize = 0;
    for (size_t i = 0; i < n; i++) {
      size_t sz = children[i].end - children[i].begin;
      if (sz <= MAX_LEAF) continue;
      if (sz > bestSize) { bestSize = sz; best = (int)i; }
    }
    if (best < 0) break;
    BRec l, r;
    split_fallback(s->prims, &children[best], &l, &r);
    l.depth = r.depth = cur->depth + 1;
    children[best] = children[n - 1];
    children[n - 1] = l;
    children[n] = r;
    n++;
  } while (n < BRANCHING);
  uint32_t node = alloc_node(s);
  for (size_t i = 0; i < n; i++) set_child(s, node, (int)i, &children[i], EMPTY_REF);
  for (size_t i = 0; i < n; i++) {
    uint32_t ref = create_large_leaf(s, bc, &children[i]);
    s->nodes[node].child[i] = ref;
  }
  return node;
}

/* recurse  bvh_builder_sah.h:222-319 */
static uint32_t recurse(OracleScene* s, BuildCtx* bc, BRec* cur) {
  const size_t N = cur->end - cur->begin;
  BSplit sp = find_split(s->prims, cur);
  const float ha = half_area3(cur->glo, cur->ghi);
  const float leafSAH = 1.0f * ha * (float)((N + (1u << LOG_BLOCK) - 1) >> LOG_BLOCK);
  const float splitSAH = 1.0f * ha + 1.0f * sp.sah;
  if (N <= MIN_LEAF || cur->depth + MIN_LARGE_LEAF_LEVELS >= MAX_DEPTH || (N <= MAX_LEAF && leafSAH <= splitSAH)) {
    deterministic_order(s->prims, cur);
    return create_large_leaf(s, bc, cur);
  }
  BRec children[BRANCHING];
  do_split(s, bc, &sp, cur, &children[0], &children[1]);
  size_t n = 2;
  while (n < BRANCHING) {
    float bestArea = -INFINITY;
    int best = -1;
    for (size_t i = 0; i < n; i++) {
      if (children[i].end - children[i].begin <= MIN_LEAF) continue;
      float a = half_area3(children[i].glo, children[i].ghi);
      if (a > bestArea) { best = (int)i; bestArea = a; }
    }
    if (best < 0) break;
    BRec l, r;
    BSplit csp = find_split(s->prims, &children[best]);
    do_split(s, bc, &csp, &children[best], &l, &r);
    l.depth = r.depth = cur->depth + 1;
    children[best] = l;
    children[n] = r;
    n++;
  }
  /* std::sort(children, greater) on prim count; for <= 16 elements libstdc++
     runs an insertion sort, which keeps equal sizes in order. */
  for (size_t i = 1; i < n; i++) {
    BRec v = children[i];
    size_t j = i;
    while (j > 0 && (v.end - v.begin) > (children[j - 1].end - children[j - 1].begin)) {
      children[j] = children[j - 1];
      j--;
    }
    children[j] = v;
  }
  uint32_t node = alloc_node(s);
  for (size_t i = 0; i < n; i++) set_child(s, node, (int)i, &children[i], EMPTY_REF);
  for (size_t i = 0; i < n; i++) {
    uint32_t ref = recurse(s, bc, &children[i]);
    s->nodes[node].child[i] = ref;
  }
  return node;
}

long orc_scene_commit(OracleScene* s) {
  free_build(s);
  qsort(s->meshes, s->nmeshes, sizeof(OMesh), cmp_mesh);
  size_t total = 0;
  for (size_t m = 0; m < s->nmeshes; m++) total += s->meshes[m].nt;
  s->prims = (OPrim*)malloc((total + 1) * sizeof(OPrim));
  size_t k = 0;
  /* createPrimRefArray  primrefgen.cpp:35-55 + scene_triangle_mesh.h:127-147,220-232 */
  for (size_t mi = 0; mi < s->nmeshes; mi++) {
    const OMesh* m = &s->meshes[mi];
    for (unsigned j = 0; j < m->nt; j++) {
      const unsigned* tri = &m->idx[3 * (size_t)j];
      if (tri[0] >= m->nv || tri[1] >= m->nv || tri[2] >= m->nv) continue;
      v3 a = mesh_vertex(m, tri[0]), b = mesh_vertex(m, tri[1]), c = mesh_vertex(m, tri[2]);
      if (!vertex_valid(a) || !vertex_valid(b) || !vertex_valid(c)) continue;
      OPrim* p = &s->prims[k++];
      p->lo[0] = fmin2(fmin2(a.x, b.x), c.x); p->hi[0] = fmax2(fmax2(a.x, b.x), c.x);
      p->lo[1] = fmin2(fmin2(a.y, b.y), c.y); p->hi[1] = fmax2(fmax2(a.y, b.y), c.y);
      p->lo[2] = fmin2(fmin2(a.z, b.z), c.z); p->hi[2] = fmax2(fmax2(a.z, b.z), c.z);
      p->geomID = m->geomID;
      p->primID = j;
    }
  }
  s->nprims = k;
  bb_empty(s->glo, s->ghi);
  s->committed = 1;
  if (k == 0) { s->root = EMPTY_REF; return 0; }
  BRec root;
  rec_init(&root, s->prims, 0, k, 1);
  for (int d = 0; d < 3; d++) { s->glo[d] = root.glo[d]; s->ghi[d] = root.ghi[d]; }
  BuildCtx bc;
  bc.tmp = (OPrim*)malloc(k * sizeof(OPrim));
  s->root = recurse(s, &bc, &root);
  free(bc.tmp);
  return (long)k;
}

/* ------------------------------------------------------------------------ */
/* statistics  kernels/bvh/bvh_statistics.cpp:10-160                       */
/* ------------------------------------------------------------------------ */

static void stats_rec(const OracleScene* s, uint32_t ref, double A, unsigned depth, OrcStats* st) {
  if (ref == EMPTY_REF) return;
  if (ref & LEAF_BIT) {
    const OLeaf* l = &s->leaves[ref & ~LEAF_BIT];
    st->num_leaves++;
    st->num_blocks += l->nblocks;
    st->leaf_sah += A * l->nblocks;
    if (depth > st->depth) st->depth = depth;
    return;
  }
  const ONode8* n = &s->nodes[ref];
  st->num_nodes++;
  st->node_sah += A;
  for (int i = 0; i < 8; i++) {
    if (n->child[i] == EMPTY_REF) continue;
    float lo[3] = {n->lo[0][i], n->lo[1][i], n->lo[2][i]};
    float hi[3] = {n->hi[0][i], n->hi[1][i], n->hi[2][i]};
    double Ai = fmax2(0.0f, half_area3(lo, hi));
    stats_rec(s, n->child[i], Ai, depth + 1, st);
  }
}

void orc_scene_stats(const OracleScene* s, OrcStats* st) {
  memset(st, 0, sizeof(*st));
  st->num_prims = s->nprims;
  for (int d = 0; d < 3; d++) { st->bounds[d] = s->glo[d]; st->bounds[3 + d] = s->ghi[d]; }
  if (s->root == EMPTY_REF) return;
  double Aroot = fmax2(0.0f, half_area3(s->glo, s->ghi));
  stats_rec(s, s->root, Aroot, 1, st);
  st->sah = Aroot > 0 ? (st->node_sah + st->leaf_sah) / Aroot : 0.0;
}

/* ------------------------------------------------------------------------ */
/* ray records                                                              */
/* ------------------------------------------------------------------------ */

typedef struct {
  v3 org, dir;
  float tnear, tfar;
} ORay;

static inline void load_ray(const char* p, ORay* r) {
  float f[12];
  memcpy(f, p, 48);
  r->org.x = f[0]; r->org.y = f[1]; r->org.z = f[2]; r->tnear = f[3];
  r->dir.x = f[4]; r->dir.y = f[5]; r->dir.z = f[6]; r->tfar = f[8];
}

typedef struct {
  int valid;
  float t, u, v;
  v3 Ng;
  unsigned geomID, primID;
} OHit;

static inline void store_hit(char* p, const OHit* h) {
  /* intersector_epilog.h:281-291 (+ instID[0] = context instID = invalid) */
  float Ng[3] = {h->Ng.x, h->Ng.y, h->Ng.z};
  unsigned inst = INVALID_ID;
  memcpy(p + 32, &h->t, 4);
  memcpy(p + 48, Ng, 12);
  memcpy(p + 60, &h->u, 4);
  memcpy(p + 64, &h->v, 4);
  memcpy(p + 68, &h->primID, 4);
  memcpy(p + 72, &h->geomID, 4);
  memcpy(p + 76, &inst, 4);
}

/* ------------------------------------------------------------------------ */
/* Moeller-Trumbore  triangle_intersector_moeller.h:62-104                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  float U, V, T, absDen;
  v3 Ng;
} MHit;

static inline int moeller(v3 v0, v3 e1, v3 e2, v3 O, v3 D, float tnear, float tfar, MHit* h) {
  const v3 C = v3sub(v0, O);
  const v3 R = cross3(C, D);
  const v3 Ng = cross3(e2, e1);
  const float den = dot3(Ng, D);
  const float absDen = fabsf(den);
  const uint32_t sgnDen = fbits(den) & 0x80000000u;
  const float U = bitsf(fbits(dot3(R, e2)) ^ sgnDen);
  const float V = bitsf(fbits(dot3(R, e1)) ^ sgnDen);
  if (!((den != 0.0f) & (U >= 0.0f) & (V >= 0.0f) & (U + V <= absDen))) return 0;
  const float T = bitsf(fbits(dot3(Ng, C)) ^ sgnDen);
  if (!((absDen * tnear < T) & (T <= absDen * tfar))) return 0;
  h->U = U; h->V = V; h->T = T; h->absDen = absDen; h->Ng = Ng;
  return 1;
}

/* stable_triangle_normal  common/math/vec3.h:210-222 */
static inline v3 stable_normal(v3 a, v3 b, v3 c) {
  const float ab_x = a.z * b.y, ab_y = a.x * b.z, ab_z = a.y * b.x;
  const float bc_x = b.z * c.y, bc_y = b.x * c.z, bc_z = b.y * c.x;
  const v3 cab = {fmaf(a.y, b.z, -ab_x), fmaf(a.z, b.x, -ab_y), fmaf(a.x, b.y, -ab_z)};
  const v3 cbc = {fmaf(b.y, c.z, -bc_x), fmaf(b.z, c.x, -bc_y), fmaf(b.x, c.y, -bc_z)};
  v3 r;
  r.x = fabsf(ab_x) < fabsf(bc_x) ? cab.x : cbc.x;
  r.y = fabsf(ab_y) < fabsf(bc_y) ? cab.y : cbc.y;
  r.z = fabsf(ab_z) < fabsf(bc_z) ? cab.z : cbc.z;
  return r;
}

typedef struct {
  float U, V, UVW, t;
  v3 Ng;
} PHit;

static inline v3 v3add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline float fmin3(float a, float b, float c) { return fmin2(fmin2(a, b), c); }
static inline float fmax3(float a, float b, float c) { return fmax2(fmax2(a, b), c); }

/* PlueckerIntersector1::intersect  kernels/geometry/triangle_intersector_pluecker.h:60-111 */
static inline int pluecker(v3 tv0, v3 tv1, v3 tv2, v3 O, v3 D, float tnear, float tfar, PHit* h) {
  const v3 v0 = v3sub(tv0, O), v1 = v3sub(tv1, O), v2 = v3sub(tv2, O);
  const v3 e0 = v3sub(v2, v0), e1 = v3sub(v0, v1), e2 = v3sub(v1, v2);
  const float U = dot3(cross3(e0, v3add(v2, v0)), D);
  const float V = dot3(cross3(e1, v3add(v0, v1)), D);
  const float W = dot3(cross3(e2, v3add(v1, v2)), D);
  const float UVW = U + V + W;
  const float eps = FLT_EPSILON * fabsf(UVW);
  if (!((fmin3(U, V, W) >= -eps) | (fmax3(U, V, W) <= eps))) return 0;
  const v3 Ng = stable_normal(e0, e1, e2);
  const float dd = dot3(Ng, D), den = dd + dd;
  const float tt = dot3(v0, Ng), T = tt + tt;
  const float t = (1.0f / den) * T;
  if (!((tnear <= t) & (t <= tfar) & (den != 0.0f))) return 0;
  h->U = U; h->V = V; h->UVW = UVW; h->t = t; h->Ng = Ng;
  return 1;
}

/* PlueckerHitM::finalize: u,v = U,V * rcp(UVW), 0 when |UVW| < min_rcp_input */
static inline void pluecker_uv(const PHit* h, float* u, float* v) {
  const float r = fabsf(h->UVW) < REF_MIN_RCP_INPUT ? 0.0f : 1.0f / h->UVW;
  *u = h->U * r;
  *v = h->V * r;
}

int orc_pluecker1(const float v0[3], const float v1[3], const float v2[3], const float org[3], const float dir[3],
                  float tnear, float tfar, float out_tuv[3], float out_Ng[3]) {
  v3 a = {v0[0], v0[1], v0[2]}, b = {v1[0], v1[1], v1[2]}, c = {v2[0], v2[1], v2[2]};
  v3 O = {org[0], org[1], org[2]}, D = {dir[0], dir[1], dir[2]};
  PHit h;
  if (!pluecker(a, b, c, O, D, tnear, tfar, &h)) return 0;
  out_tuv[0] = h.t;
  pluecker_uv(&h, &out_tuv[1], &out_tuv[2]);
  out_Ng[0] = h.Ng.x; out_Ng[1] = h.Ng.y; out_Ng[2] = h.Ng.z;
  return 1;
}

int orc_moeller1(const float v0[3], const float v1[3], const float v2[3], const float org[3], const float dir[3],
                 float tnear, float tfar, float out_UVTden[4], float out_tuv[3], float out_Ng[3]) {
  v3 a = {v0[0], v0[1], v0[2]}, b = {v1[0], v1[1], v1[2]}, c = {v2[0], v2[1], v2[2]};
  v3 O = {org[0], org[1], org[2]}, D = {dir[0], dir[1], dir[2]};
  MHit h;
  if (!moeller(a, v3sub(a, b), v3sub(c, a), O, D, tnear, tfar, &h)) return 0;
  const float rcp = 1.0f / h.absDen;
  out_UVTden[0] = h.U; out_UVTden[1] = h.V; out_UVTden[2] = h.T; out_UVTden[3] = h.absDen;
  out_tuv[0] = h.T * rcp; out_tuv[1] = h.U * rcp; out_tuv[2] = h.V * rcp;
  out_Ng[0] = h.Ng.x; out_Ng[1] = h.Ng.y; out_Ng[2] = h.Ng.z;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* traversal  bvh_intersector1.cpp:30-195, node_intersector1.h             */
/* ------------------------------------------------------------------------ */

typedef struct { uint64_t nodes, leaves, tris; } OCount;

static uint64_t g_counters[3];
static pthread_mutex_t g_counter_lock = PTHREAD_MUTEX_INITIALIZER;

void orc_counters(uint64_t out[3]) {
  pthread_mutex_lock(&g_counter_lock);
  out[0] = g_counters[0]; out[1] = g_counters[1]; out[2] = g_counters[2];
  pthread_mutex_unlock(&g_counter_lock);
}

typedef struct {
  v3 org, rdir, org_rdir;
  v3 rdir_near, rdir_far;  /* robust: 1/d scaled by (1 -+ 3 ulp) */
  int nearX, nearY, nearZ; /* 0: lower plane is near, 1: upper */
  int robust;
  float tnear, tfar;       /* clamped to >= 0 */
} TravRay;

/* rcp_safe = rcp(zero_fix(d)), zero_fix: |d| < 1e-18 -> +1e-18 (vec3fa.h:172-177) */
static inline float rcp_safe(float d) {
  if (fabsf(d) < REF_MIN_RCP_INPUT) d = REF_MIN_RCP_INPUT;
  return 1.0f / d;
}

static inline float zero_fix(float d) { return fabsf(d) < REF_MIN_RCP_INPUT ? REF_MIN_RCP_INPUT : d; }

static inline void trav_init(TravRay* t, const ORay* r, int robust) {
  t->robust = robust;
  if (robust) {
    /* TravRayBase<N,Nx,true>  node_intersector1.h:122-153 */
    const float round_down = 1.0f - 3.0f * FLT_EPSILON, round_up = 1.0f + 3.0f * FLT_EPSILON;
    const v3 rd = {1.0f / zero_fix(r->dir.x), 1.0f / zero_fix(r->dir.y), 1.0f / zero_fix(r->dir.z)};
    t->rdir_near.x = round_down * rd.x; t->rdir_near.y = round_down * rd.y; t->rdir_near.z = round_down * rd.z;
    t->rdir_far.x = round_up * rd.x; t->rdir_far.y = round_up * rd.y; t->rdir_far.z = round_up * rd.z;
  }
  t->org = r->org;
  t->rdir.x = rcp_safe(r->dir.x);
  t->rdir.y = rcp_safe(r->dir.y);
  t->rdir.z = rcp_safe(r->dir.z);
  t->org_rdir = v3mul(r->org, t->rdir);
  if (robust) {
    t->nearX = t->rdir_near.x >= 0.0f ? 0 : 1;
    t->nearY = t->rdir_near.y >= 0.0f ? 0 : 1;
    t->nearZ = t->rdir_near.z >= 0.0f ? 0 : 1;
  } else {
    t->nearX = t->rdir.x >= 0.0f ? 0 : 1;
    t->nearY = t->rdir.y >= 0.0f ? 0 : 1;
    t->nearZ = t->rdir.z >= 0.0f ? 0 : 1;
  }
  t->tnear = fmax2(r->tnear, 0.0f);
  t->tfar = fmax2(r->tfar, 0.0f);
}

/* intersectNode<8,8>: t = msub(plane, rdir, org_rdir)  node_intersector1.h:527-585 */
static inline unsigned node_test(const ONode8* n, const TravRay* t, float dist[8]) {
  const float* nx = t->nearX ? n->hi[0] : n->lo[0];
  const float* fx = t->nearX ? n->lo[0] : n->hi[0];
  const float* ny = t->nearY ? n->hi[1] : n->lo[1];
  const float* fy = t->nearY ? n->lo[1] : n->hi[1];
  const float* nz = t->nearZ ? n->hi[2] : n->lo[2];
  const float* fz = t->nearZ ? n->lo[2] : n->hi[2];
  unsigned mask = 0;
  if (t->robust) {
    /* intersectNodeRobust  node_intersector1.h:622-637 */
    for (int i = 0; i < 8; i++) {
      float tNx = (nx[i] - t->org.x) * t->rdir_near.x;
      float tNy = (ny[i] - t->org.y) * t->rdir_near.y;
      float tNz = (nz[i] - t->org.z) * t->rdir_near.z;
      float tFx = (fx[i] - t->org.x) * t->rdir_far.x;
      float tFy = (fy[i] - t->org.y) * t->rdir_far.y;
      float tFz = (fz[i] - t->org.z) * t->rdir_far.z;
      float tN = fmax2(fmax2(tNx, tNy), fmax2(tNz, t->tnear));
      float tF = fmin2(fmin2(tFx, tFy), fmin2(tFz, t->tfar));
      dist[i] = tN;
      mask |= (unsigned)(tN <= tF) << i;
    }
    return mask;
  }
  for (int i = 0; i < 8; i++) {
    float tNx = fmaf(nx[i], t->rdir.x, -t->org_rdir.x);
    float tNy = fmaf(ny[i], t->rdir.y, -t->org_rdir.y);
    float tNz = fmaf(nz[i], t->rdir.z, -t->org_rdir.z);
    float tFx = fmaf(fx[i], t->rdir.x, -t->org_rdir.x);
    float tFy = fmaf(fy[i], t->rdir.y, -t->org_rdir.y);
    float tFz = fmaf(fz[i], t->rdir.z, -t->org_rdir.z);
    float tN = fmax2(fmax2(tNx, tNy), fmax2(tNz, t->tnear));
    float tF = fmin2(fmin2(tFx, tFy), fmin2(tFz, t->tfar));
    dist[i] = tN;
    mask |= (unsigned)(tN <= tF) << i;
  }
  return mask;
}

/* One Triangle4 block: all lanes against the same tfar, then the nearest
   valid lane (lowest lane on ties, vfloat4_sse2.h:887-892) is committed.
   With a filter callback (Intersect1EpilogM, intersector_epilog.h:237-276) the
   nearest lane is offered to it: a rejected lane is dropped and the next
   nearest offered; an accepted one is committed, tfar becomes its distance and
   the lanes at that distance or nearer are still offered. */
static inline int leaf_block_closest(const OTri4* tri, const ORay* r, float tfar_now, OHit* hit, OCount* cnt,
                                     int robust, orc_filter_fn filter, void* fuser) {
  int valid[4];
  float tv[4];
  MHit h[4];
  PHit ph[4];
  int any = 0;
  for (int i = 0; i < 4; i++) {
    valid[i] = 0;
    tv[i] = INFINITY;
    if (tri->geomID[i] == INVALID_ID) continue;
    cnt->tris++;
    v3 a = {tri->v0[0][i], tri->v0[1][i], tri->v0[2][i]};
    v3 b = {tri->e1[0][i], tri->e1[1][i], tri->e1[2][i]};
    v3 c = {tri->e2[0][i], tri->e2[1][i], tri->e2[2][i]};
    if (robust) {
      valid[i] = pluecker(a, b, c, r->org, r->dir, r->tnear, tfar_now, &ph[i]);
      if (valid[i]) tv[i] = ph[i].t;
    } else {
      valid[i] = moeller(a, b, c, r->org, r->dir, r->tnear, tfar_now, &h[i]);
      if (valid[i]) tv[i] = h[i].T * (1.0f / h[i].absDen);
    }
    any |= valid[i];
  }
  if (!any) return 0;
  int found = 0;
  for (;;) {
    if (!(valid[0] | valid[1] | valid[2] | valid[3])) return found;
    float best = INFINITY;
    for (int i = 0; i < 4; i++)
      if (valid[i] && tv[i] < best) best = tv[i];
    int sel = -1;
    for (int i = 0; i < 4 && sel < 0; i++)
      if (valid[i] && tv[i] == best) sel = i;
    if (sel < 0)
      for (int i = 0; i < 4 && sel < 0; i++)
        if (valid[i]) sel = i;
    OHit c;
    c.valid = 1;
    if (robust) {
      c.t = ph[sel].t;
      pluecker_uv(&ph[sel], &c.u, &c.v);
      c.Ng = ph[sel].Ng;
    } else {
      const float rcp = 1.0f / h[sel].absDen;
      c.t = h[sel].T * rcp;
      c.u = h[sel].U * rcp;
      c.v = h[sel].V * rcp;
      c.Ng = h[sel].Ng;
    }
    c.geomID = tri->geomID[sel];
    c.primID = tri->primID[sel];
    if (!filter) {
      *hit = c;
      return 1;
    }
    valid[sel] = 0;
    if (!filter(fuser, c.geomID, c.primID, c.u, c.v, c.t)) continue;
    *hit = c;
    found = 1;
    for (int i = 0; i < 4; i++) valid[i] &= tv[i] <= c.t;
  }
}

/* With a filter callback (Occluded1EpilogM, intersector_epilog.h:397-435) the
   hit lanes are offered to it in lane order until one is accepted. */
static inline int leaf_block_any(const OTri4* tri, const ORay* r, OCount* cnt, int robust, orc_filter_fn filter,
                                 void* fuser) {
  for (int i = 0; i < 4; i++) {
    if (tri->geomID[i] == INVALID_ID) continue;
    cnt->tris++;
    v3 a = {tri->v0[0][i], tri->v0[1][i], tri->v0[2][i]};
    v3 b = {tri->e1[0][i], tri->e1[1][i], tri->e1[2][i]};
    v3 c = {tri->e2[0][i], tri->e2[1][i], tri->e2[2][i]};
    float t, u, v;
    if (robust) {
      PHit h;
      if (!pluecker(a, b, c, r->org, r->dir, r->tnear, r->tfar, &h)) continue;
      t = h.t;
      pluecker_uv(&h, &u, &v);
    } else {
      MHit h;
      if (!moeller(a, b, c, r->org, r->dir, r->tnear, r->tfar, &h)) continue;
      const float rcp = 1.0f / h.absDen;
      t = h.T * rcp;
      u = h.U * rcp;
      v = h.V * rcp;
    }
    if (!filter || filter(fuser, tri->geomID[i], tri->primID[i], u, v, t)) return 1;
  }
  return 0;
}

#define STACK_SIZE 1024

typedef struct { uint32_t ref; float dist; } SItem;

static void trace_closest(const OracleScene* s, char* rec, OCount* cnt) {
  ORay r;
  load_ray(rec, &r);
  /* stream filter: only rays with tnear <= tfar are traced */
  if (!(r.tnear <= r.tfar)) return;
  if (s->root == EMPTY_REF) return;
  TravRay t;
  trav_init(&t, &r, s->robust);
  OHit hit;
  memset(&hit, 0, sizeof(hit));
  hit.valid = 0;
  SItem stack[STACK_SIZE];
  int sp = 0;
  stack[sp].ref = s->root;
  stack[sp].dist = -INFINITY;
  sp++;
  while (sp > 0) {
    sp--;
    uint32_t cur = stack[sp].ref;
    if (stack[sp].dist > r.tfar) continue;
    while (!(cur & LEAF_BIT)) {
      const ONode8* n = &s->nodes[cur];
      float dist[8];
      cnt->nodes++;
      unsigned mask = node_test(n, &t, dist);
      if (!mask) { cur = EMPTY_REF; break; }
      /* closest child first, the others pushed far-to-near */
      SItem hits[8];
      int nh = 0;
      for (int i = 0; i < 8; i++) {
        if (!(mask >> i & 1)) continue;
        SItem it = {n->child[i], dist[i]};
        int j = nh++;
        while (j > 0 && hits[j - 1].dist > it.dist) { hits[j] = hits[j - 1]; j--; }
        hits[j] = it;
      }
      for (int k = nh - 1; k >= 1; k--) {
        if (sp < STACK_SIZE) stack[sp++] = hits[k];
      }
      cur = hits[0].ref;
    }
    if (cur == EMPTY_REF) continue;
    cnt->leaves++;
    const OLeaf* lf = &s->leaves[cur & ~LEAF_BIT];
    for (uint32_t b = 0; b < lf->nblocks; b++) {
      if (leaf_block_closest(&s->tris[lf->first + b], &r, r.tfar, &hit, cnt, s->robust, s->ifilter, s->filter_user))
        r.tfar = hit.t;
    }
    t.tfar = r.tfar;
  }
  if (hit.valid) store_hit(rec, &hit);
}

static void trace_occluded(const OracleScene* s, char* rec, OCount* cnt) {
  ORay r;
  load_ray(rec, &r);
  /* bvh_intersector_stream_filters.cpp:75: skip invalid / already occluded */
  if (r.tnear > r.tfar || r.tfar < 0.0f) return;
  if (!(r.tnear <= r.tfar)) return;
  if (s->root == EMPTY_REF) return;
  TravRay t;
  trav_init(&t, &r, s->robust);
  uint32_t stack[STACK_SIZE];
  int sp = 0;
  stack[sp++] = s->root;
  while (sp > 0) {
    uint32_t cur = stack[--sp];
    while (!(cur & LEAF_BIT)) {
      const ONode8* n = &s->nodes[cur];
      float dist[8];
      cnt->nodes++;
      unsigned mask = node_test(n, &t, dist);
      if (!mask) { cur = EMPTY_REF; break; }
      int first = __builtin_ctz(mask);
      mask &= mask - 1;
      while (mask) {
        int i = 31 - __builtin_clz(mask);
        mask &= ~(1u << i);
        if (sp < STACK_SIZE) stack[sp++] = n->child[i];
      }
      cur = n->child[first];
    }
    if (cur == EMPTY_REF) continue;
    cnt->leaves++;
    const OLeaf* lf = &s->leaves[cur & ~LEAF_BIT];
    for (uint32_t b = 0; b < lf->nblocks; b++) {
      if (leaf_block_any(&s->tris[lf->first + b], &r, cnt, s->robust, s->ofilter, s->filter_user)) {
        float ninf = -INFINITY;
        memcpy(rec + 32, &ninf, 4);
        return;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* multithreaded stream driver                                              */
/* ------------------------------------------------------------------------ */

typedef struct {
  const OracleScene* s;
  char* rays;
  unsigned M;
  size_t stride;
  int occluded;
  volatile unsigned next;
} Job;

#define CHUNK 256

static void* worker(void* arg) {
  Job* j = (Job*)arg;
  OCount cnt = {0, 0, 0};
  for (;;) {
    unsigned b = __atomic_fetch_add((unsigned*)&j->next, CHUNK, __ATOMIC_RELAXED);
    if (b >= j->M) break;
    unsigned e = b + CHUNK < j->M ? b + CHUNK : j->M;
    for (unsigned i = b; i < e; i++) {
      char* rec = j->rays + (size_t)i * j->stride;
      if (j->occluded) trace_occluded(j->s, rec, &cnt);
      else trace_closest(j->s, rec, &cnt);
    }
  }
  pthread_mutex_lock(&g_counter_lock);
  g_counters[0] += cnt.nodes;
  g_counters[1] += cnt.leaves;
  g_counters[2] += cnt.tris;
  pthread_mutex_unlock(&g_counter_lock);
  return NULL;
}

static void run_stream(const OracleScene* s, void* rays, unsigned M, size_t stride, int nthreads, int occluded) {
  pthread_mutex_lock(&g_counter_lock);
  g_counters[0] = g_counters[1] = g_counters[2] = 0;
  pthread_mutex_unlock(&g_counter_lock);
  if (nthreads <= 0) nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (nthreads < 1) nthreads = 1;
  if ((unsigned)nthreads > M / CHUNK + 1) nthreads = (int)(M / CHUNK + 1);
  Job j = {s, (char*)rays, M, stride, occluded, 0};
  if (nthreads == 1) { worker(&j); return; }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, worker, &j);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  free(th);
}

void orc_intersect1M(const OracleScene* s, void* rays, unsigned M, size_t stride, int nthreads) {
  run_stream(s, rays, M, stride, nthreads, 0);
}

void orc_occluded1M(const OracleScene* s, void* rays, unsigned M, size_t stride, int nthreads) {
  run_stream(s, rays, M, stride, nthreads, 1);
}

/* ---- instances (RTC_GEOMETRY_TYPE_INSTANCE, one level) ----------------------
   kernels/geometry/instance_intersector.cpp:56-97: the ray is moved into the
   instance's space (xfmPoint / xfmVector, common/math/affinespace.h:102-103,
   madd chains), traced in the instanced scene with the current tfar, and its
   world origin and direction are restored; the hit keeps the instanced
   scene's geomID / primID / object-space Ng and gets instID = the instance's
   geometry ID.  The world-to-local map is rcp(AffineSpace3fa)
   (affinespace.h:83, linearspace3.h:44-50: transposed adjoint / det,
   -(inverse * p)) with the correctly rounded 1/det. */

static int orc_invert(const float* m, float* o) {
  const v3 vx = {m[0], m[1], m[2]}, vy = {m[3], m[4], m[5]}, vz = {m[6], m[7], m[8]};
  const v3 c0 = cross3(vy, vz), c1 = cross3(vz, vx), c2 = cross3(vx, vy);
  const float det = dot3(vx, c0);
  if (!(det != 0.0f) || !isfinite(det)) return 0;
  const float r = 1.0f / det;
  const float c[3][3] = {{c0.x, c0.y, c0.z}, {c1.x, c1.y, c1.z}, {c2.x, c2.y, c2.z}};
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) o[3 * j + i] = c[i][j] * r;
  for (int k = 0; k < 3; k++)
    o[9 + k] = -fmaf(m[9], o[k], fmaf(m[10], o[3 + k], m[11] * o[6 + k]));
  for (int k = 0; k < 12; k++)
    if (!isfinite(o[k])) return 0;
  return 1;
}

static void to_instance(const float* w, const char* rec, char* tmp) {
  float f[12];
  memcpy(f, rec, sizeof(f));
  float o[3], d[3];
  for (int c = 0; c < 3; c++) {
    o[c] = fmaf(f[0], w[c], fmaf(f[1], w[3 + c], fmaf(f[2], w[6 + c], w[9 + c])));
    d[c] = fmaf(f[4], w[c], fmaf(f[5], w[3 + c], f[6] * w[6 + c]));
  }
  memcpy(tmp, rec, 80);
  memcpy(tmp + 0, o, 12);
  memcpy(tmp + 16, d, 12);
}

void orc_intersect_instanced(const OracleScene* top, unsigned ninst, const OracleScene* const* scenes,
                             const float* l2w, const unsigned* inst_geomIDs, void* rays, unsigned M, size_t stride) {
  float* w2l = (float*)malloc(sizeof(float) * 12 * (ninst ? ninst : 1));
  int* ok = (int*)malloc(sizeof(int) * (ninst ? ninst : 1));
  for (unsigned k = 0; k < ninst; k++) ok[k] = orc_invert(l2w + 12 * k, w2l + 12 * k);
  OCount cnt = {0, 0, 0};
  for (unsigned i = 0; i < M; i++) {
    char* rec = (char*)rays + (size_t)i * stride;
    ORay r;
    load_ray(rec, &r);
    if (!(r.tnear <= r.tfar)) continue;
    if (top) trace_closest(top, rec, &cnt);
    for (unsigned k = 0; k < ninst; k++) {
      if (!ok[k] || scenes[k]->root == EMPTY_REF) continue;
      char tmp[80];
      to_instance(w2l + 12 * k, rec, tmp);
      const uint32_t none = 0xFFFFFFFFu;
      memcpy(tmp + 72, &none, 4);
      trace_closest(scenes[k], tmp, &cnt);
      uint32_t g;
      memcpy(&g, tmp + 72, 4);
      if (g == none) continue;
      memcpy(rec + 32, tmp + 32, 4);        /* tfar */
      memcpy(rec + 48, tmp + 48, 28);       /* Ng, u, v, primID, geomID */
      memcpy(rec + 76, &inst_geomIDs[k], 4); /* instID[0] */
    }
  }
  free(w2l);
  free(ok);
}

void orc_occluded_instanced(const OracleScene* top, unsigned ninst, const OracleScene* const* scenes,
                            const float* l2w, void* rays, unsigned M, size_t stride) {
  float* w2l = (float*)malloc(sizeof(float) * 12 * (ninst ? ninst : 1));
  int* ok = (int*)malloc(sizeof(int) * (ninst ? ninst : 1));
  for (unsigned k = 0; k < ninst; k++) ok[k] = orc_invert(l2w + 12 * k, w2l + 12 * k);
  OCount cnt = {0, 0, 0};
  for (unsigned i = 0; i < M; i++) {
    char* rec = (char*)rays + (size_t)i * stride;
    ORay r;
    load_ray(rec, &r);
    if (r.tnear > r.tfar || r.tfar < 0.0f || !(r.tnear <= r.tfar)) continue;
    if (top) trace_occluded(top, rec, &cnt);
    float tf;
    memcpy(&tf, rec + 32, 4);
    for (unsigned k = 0; k < ninst && !(tf < 0.0f); k++) {
      if (!ok[k] || scenes[k]->root == EMPTY_REF) continue;
      char tmp[80];
      to_instance(w2l + 12 * k, rec, tmp);
      trace_occluded(scenes[k], tmp, &cnt);
      float t2;
      memcpy(&t2, tmp + 32, 4);
      if (t2 < 0.0f) {
        memcpy(rec + 32, &t2, 4);
        tf = t2;
      }
    }
  }
  free(w2l);
  free(ok);
}

/* ------------------------------------------------------------------------ */
/* brute force                                                              */
/* ------------------------------------------------------------------------ */

/* the leaf values of one primitive: (v0, e1, e2), or (v0, v1, v2) when robust */
static int prim_tri(const OracleScene* s, unsigned geomID, unsigned primID, v3* v0, v3* e1, v3* e2) {
  const OMesh* m = find_mesh(s, geomID);
  if (!m || primID >= m->nt) return 0;
  const unsigned* tri = &m->idx[3 * (size_t)primID];
  if (tri[0] >= m->nv || tri[1] >= m->nv || tri[2] >= m->nv) return 0;
  v3 p0 = mesh_vertex(m, tri[0]), p1 = mesh_vertex(m, tri[1]), p2 = mesh_vertex(m, tri[2]);
  *v0 = p0;
  *e1 = s->robust ? p1 : v3sub(p0, p1);
  *e2 = s->robust ? p2 : v3sub(p2, p0);
  return 1;
}

void orc_brute_intersect1M(const OracleScene* s, void* rays, unsigned M, size_t stride) {
  for (unsigned i = 0; i < M; i++) {
    char* rec = (char*)rays + (size_t)i * stride;
    ORay r;
    load_ray(rec, &r);
    if (!(r.tnear <= r.tfar)) continue;
    OHit hit;
    memset(&hit, 0, sizeof(hit));
    hit.valid = 0;
    for (size_t k = 0; k < s->nprims; k++) {
      v3 v0, e1, e2;
      if (!prim_tri(s, s->prims[k].geomID, s->prims[k].primID, &v0, &e1, &e2)) continue;
      if (s->robust) {
        PHit h;
        if (!pluecker(v0, e1, e2, r.org, r.dir, r.tnear, r.tfar, &h)) continue;
        hit.valid = 1;
        hit.t = h.t;
        pluecker_uv(&h, &hit.u, &hit.v);
        hit.Ng = h.Ng;
      } else {
        MHit h;
        if (!moeller(v0, e1, e2, r.org, r.dir, r.tnear, r.tfar, &h)) continue;
        const float rcp = 1.0f / h.absDen;
        hit.valid = 1;
        hit.t = h.T * rcp;
        hit.u = h.U * rcp;
        hit.v = h.V * rcp;
        hit.Ng = h.Ng;
      }
      hit.geomID = s->prims[k].geomID;
      hit.primID = s->prims[k].primID;
      r.tfar = hit.t;
    }
    if (hit.valid) store_hit(rec, &hit);
  }
}

void orc_brute_occluded1M(const OracleScene* s, void* rays, unsigned M, size_t stride) {
  for (unsigned i = 0; i < M; i++) {
    char* rec = (char*)rays + (size_t)i * stride;
    ORay r;
    load_ray(rec, &r);
    if (r.tnear > r.tfar || r.tfar < 0.0f || !(r.tnear <= r.tfar)) continue;
    for (size_t k = 0; k < s->nprims; k++) {
      v3 v0, e1, e2;
      if (!prim_tri(s, s->prims[k].geomID, s->prims[k].primID, &v0, &e1, &e2)) continue;
      MHit h;
      PHit ph;
      if (s->robust ? pluecker(v0, e1, e2, r.org, r.dir, r.tnear, r.tfar, &ph)
                    : moeller(v0, e1, e2, r.org, r.dir, r.tnear, r.tfar, &h)) {
        float ninf = -INFINITY;
        memcpy(rec + 32, &ninf, 4);
        break;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* FP64 adjudication                                                        */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y, z; } d3;
static inline d3 dsub(d3 a, d3 b) { d3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 dcross(d3 a, d3 b) {
  d3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}

/* returns 1 hit, 0 miss, -1 degenerate; u,v are the reference's barycentrics
   (hit = v0 + u (v1-v0) + v (v2-v0)) */
static int hit64(const OracleScene* s, const ORay* r, unsigned g, unsigned p, double* t, double* u, double* v) {
  const OMesh* m = find_mesh(s, g);
  if (!m || p >= m->nt) return -1;
  const unsigned* tri = &m->idx[3 * (size_t)p];
  if (tri[0] >= m->nv || tri[1] >= m->nv || tri[2] >= m->nv) return -1;
  v3 a = mesh_vertex(m, tri[0]), b = mesh_vertex(m, tri[1]), c = mesh_vertex(m, tri[2]);
  d3 v0 = {a.x, a.y, a.z}, v1 = {b.x, b.y, b.z}, v2 = {c.x, c.y, c.z};
  d3 O = {r->org.x, r->org.y, r->org.z}, D = {r->dir.x, r->dir.y, r->dir.z};
  d3 e1 = dsub(v1, v0), e2 = dsub(v2, v0);
  d3 P = dcross(D, e2);
  double det = ddot(e1, P);
  double scale = sqrt(ddot(e1, e1) * ddot(e2, e2) * ddot(D, D));
  if (!(fabs(det) > 1e-14 * scale)) return -1;
  double inv = 1.0 / det;
  d3 Tv = dsub(O, v0);
  *u = ddot(Tv, P) * inv;
  d3 Q = dcross(Tv, e1);
  *v = ddot(D, Q) * inv;
  *t = ddot(e2, Q) * inv;
  return (*u >= 0 && *v >= 0 && *u + *v <= 1 && *t > 0) ? 1 : 0;
}

int orc_fp64_hit(const OracleScene* s, const void* rayhit_in, unsigned geomID, unsigned primID, double* t, double* u,
                 double* v) {
  ORay r;
  load_ray((const char*)rayhit_in, &r);
  return hit64(s, &r, geomID, primID, t, u, v) == 1;
}

int orc_fp32_hit(const OracleScene* s, const void* rayhit_in, unsigned geomID, unsigned primID, float* t) {
  ORay r;
  load_ray((const char*)rayhit_in, &r);
  const OMesh* m = find_mesh(s, geomID);
  if (!m || primID >= m->nt) return 0;
  const unsigned* tri = &m->idx[3 * (size_t)primID];
  if (tri[0] >= m->nv || tri[1] >= m->nv || tri[2] >= m->nv) return 0;
  const v3 p0 = mesh_vertex(m, tri[0]), p1 = mesh_vertex(m, tri[1]), p2 = mesh_vertex(m, tri[2]);
  if (s->robust) {
    PHit h;
    if (!pluecker(p0, p1, p2, r.org, r.dir, r.tnear, r.tfar, &h)) return 0;
    *t = h.t;
    return 1;
  }
  MHit h;
  if (!moeller(p0, v3sub(p0, p1), v3sub(p2, p0), r.org, r.dir, r.tnear, r.tfar, &h)) return 0;
  *t = h.T * (1.0f / h.absDen);
  return 1;
}

static inline int grazing(double u, double v) {
  const double e = 1e-6;
  return fabs(u) < e || fabs(v) < e || fabs(1.0 - u - v) < e;
}

static inline double ulp32(double t) {
  float f = (float)fabs(t);
  return (double)nextafterf(f, INFINITY) - (double)f;
}

int orc_adjudicate(const OracleScene* s, const void* rayhit_in, unsigned gA, unsigned pA, float tA, unsigned gB,
                   unsigned pB, float tB, int tie_ulps) {
  (void)tA; (void)tB;
  ORay r;
  load_ray((const char*)rayhit_in, &r);
  double ta = 0, ua = 0, va = 0, tb = 0, ub = 0, vb = 0;
  int ha = -2, hb = -2;
  if (gA != INVALID_ID) ha = hit64(s, &r, gA, pA, &ta, &ua, &va);
  if (gB != INVALID_ID) hb = hit64(s, &r, gB, pB, &tb, &ub, &vb);
  /* a crossing outside the ray's (tnear, tfar] interval is not a hit; one
     within a relative 1e-6 of either end is a boundary (grazing) case */
  const double lo = r.tnear > 0 ? r.tnear : 0.0, hi = r.tfar;
  int edgeA = 0, edgeB = 0;
  if (ha == 1) {
    if (fabs(ta - lo) <= 1e-6 * (fabs(lo) + 1e-30) || (isfinite(hi) && fabs(ta - hi) <= 1e-6 * fabs(hi))) edgeA = 1;
    if (!(ta > lo && ta <= hi)) ha = 0;
  }
  if (hb == 1) {
    if (fabs(tb - lo) <= 1e-6 * (fabs(lo) + 1e-30) || (isfinite(hi) && fabs(tb - hi) <= 1e-6 * fabs(hi))) edgeB = 1;
    if (!(tb > lo && tb <= hi)) hb = 0;
  }
  int grazeA = (ha == -1) || edgeA || (ha >= 0 && gA != INVALID_ID && grazing(ua, va));
  int grazeB = (hb == -1) || edgeB || (hb >= 0 && gB != INVALID_ID && grazing(ub, vb));
  if (ha == 1 && hb == 1) {
    double tol = tie_ulps * ulp32(ta > tb ? ta : tb);
    if (fabs(ta - tb) <= tol) return 1;
    if (grazeA || grazeB) return 2;
    return ta < tb ? 3 : 4;
  }
  if (grazeA || grazeB) return 2;
  if (ha == 1 && hb != 1) return 3;
  if (hb == 1 && ha != 1) return 4;
  return 0;
}
