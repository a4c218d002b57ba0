/*
 * Oracle (test infrastructure only): C restatement of the reference's sparse
 * voxel octree build.  It checks the GPU builder on the GPU machine, where the
 * reference sources are absent; in this container it is itself checked
 * against golden SVO files produced by the reference's own builder.
 *
 *   construct / insert / build    src/model/OctreeConstruction.h:75-194
 *   octree side                   src/model/OctreeConstruction.h:197-223
 *   HashCache (--dag)             src/model/OctreeConstruction.h:19-30
 *   ChannelDiffHeuristic          src/model/OctreeConstruction.h:32-39, Grid.cpp:81-137
 *   StdDevHeuristic               src/model/OctreeConstruction.h:41-48, Grid.cpp:139-214
 *   find / generate_ropes         src/model/Octree.cpp:116-201
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "xo.h"

typedef struct {
    uint32_t children[8];
    uint32_t color;
    uint32_t is_leaf_depth;
} Node;

#define LEAF 0x80000000u

typedef struct {
    Node* v;
    uint64_t n, cap;
} NodeVec;

typedef struct {
    uint64_t* slots; /* index+1 into the node vector, 0 = empty */
    uint64_t mask;
    uint64_t used;
} Cache;

typedef struct {
    const uint8_t* rgba;
    uint64_t dim[3];
    int heuristic;
    double threshold;
    int dag;
    NodeVec nodes;
    Cache cache;
    xo_build_stats* stats;
    int oom;
} Builder;

static int push_node(NodeVec* v, const Node* n) {
    if (v->n == v->cap) {
        uint64_t cap = v->cap ? v->cap * 2 : 1024;
        Node* p = (Node*)realloc(v->v, cap * sizeof(Node));
        if (!p) return -1;
        v->v = p;
        v->cap = cap;
    }
    v->v[v->n++] = *n;
    return 0;
}

static uint64_t node_hash(const Node* n) {
    uint64_t h = 1469598103934665603ull;
    const uint32_t* w = (const uint32_t*)n;
    for (int i = 0; i < 10; ++i) {
        h ^= w[i];
        h *= 1099511628211ull;
        h ^= h >> 29;
    }
    return h;
}

static int cache_grow(Builder* b) {
    uint64_t cap = b->cache.mask ? (b->cache.mask + 1) * 2 : 4096;
    uint64_t* s = (uint64_t*)calloc(cap, sizeof(uint64_t));
    if (!s) return -1;
    for (uint64_t i = 0; b->cache.slots && i <= b->cache.mask; ++i) {
        uint64_t e = b->cache.slots[i];
        if (!e) continue;
        uint64_t h = node_hash(&b->nodes.v[e - 1]) & (cap - 1);
        while (s[h]) h = (h + 1) & (cap - 1);
        s[h] = e;
    }
    free(b->cache.slots);
    b->cache.slots = s;
    b->cache.mask = cap - 1;
    return 0;
}

/* OctreeBuilder::insert (OctreeConstruction.h:75-90) with HashCache or
 * NoopCache: returns the index of an equal node inserted earlier, else
 * appends. */
static uint32_t insert(Builder* b, const Node* node, int leaf) {
    uint32_t end_index = (uint32_t)b->nodes.n;
    uint32_t actual = end_index;
    if (b->dag) {
        if ((b->cache.used + 1) * 2 > b->cache.mask + 1 && cache_grow(b)) { b->oom = 1; return 0; }
        uint64_t h = node_hash(node) & b->cache.mask;
        for (;;) {
            uint64_t e = b->cache.slots[h];
            if (!e) {
                b->cache.slots[h] = (uint64_t)end_index + 1;
                b->cache.used++;
                break;
            }
            if (memcmp(&b->nodes.v[e - 1], node, sizeof(Node)) == 0) {
                actual = (uint32_t)(e - 1);
                break;
            }
            h = (h + 1) & b->cache.mask;
        }
    }
    int inserted = actual == end_index;
    if (inserted && push_node(&b->nodes, node)) { b->oom = 1; return 0; }
    b->stats->total_nodes++;
    if (leaf) {
        b->stats->total_leaves++;
        if (inserted) b->stats->unique_leaves++;
    }
    return actual;
}

static inline uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

/* Grid::vol_scan (Grid.cpp:81-137) and Grid::stddev_scan (Grid.cpp:139-214):
 * returns the packed average colour and whether the heuristic splits. */
static void grid_scan(const Builder* b, const uint64_t off[3], uint64_t extent, uint32_t* avg_out,
                      int* split_out) {
    uint64_t lo[3], hi[3];
    for (int i = 0; i < 3; ++i) {
        lo[i] = umin64(b->dim[i], off[i]);
        hi[i] = umin64(b->dim[i], off[i] + extent);
    }
    uint64_t n = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
    if (n == 0) {
        *avg_out = 0;
        *split_out = b->heuristic == XO_HEUR_CHANNEL_DIFF ? (0 > (int)b->threshold) : (0.0 > b->threshold);
        return;
    }
    uint64_t acc[4] = {0, 0, 0, 0};
    uint8_t mn[4] = {255, 255, 255, 255}, mx[4] = {0, 0, 0, 0};
    for (uint64_t z = lo[2]; z < hi[2]; ++z)
        for (uint64_t y = lo[1]; y < hi[1]; ++y) {
            const uint8_t* row = b->rgba + 4 * (z * b->dim[0] * b->dim[1] + y * b->dim[0]);
            for (uint64_t x = lo[0]; x < hi[0]; ++x) {
                const uint8_t* p = row + 4 * x;
                for (int c = 0; c < 4; ++c) {
                    acc[c] += p[c];
                    if (p[c] < mn[c]) mn[c] = p[c];
                    if (p[c] > mx[c]) mx[c] = p[c];
                }
            }
        }
    if (b->heuristic == XO_HEUR_CHANNEL_DIFF) {
        uint32_t avg = 0;
        int maxdiff = 0;
        for (int c = 0; c < 4; ++c) {
            avg |= (uint32_t)(uint8_t)(acc[c] / n) << (8 * c);
            int d = (int)mx[c] - (int)mn[c]; /* _mm_subs_epu8 saturates at 0 */
            if (d < 0) d = 0;
            if (d > maxdiff) maxdiff = d;
        }
        *avg_out = avg;
        *split_out = maxdiff > (int)(uint8_t)b->threshold;
        return;
    }
    double nd = (double)n;
    double av[4];
    uint32_t avg = 0;
    for (int c = 0; c < 4; ++c) {
        av[c] = (double)acc[c] / nd;
        avg |= (uint32_t)(uint8_t)av[c] << (8 * c);
    }
    double s = 0;
    for (uint64_t z = lo[2]; z < hi[2]; ++z)
        for (uint64_t y = lo[1]; y < hi[1]; ++y) {
            const uint8_t* row = b->rgba + 4 * (z * b->dim[0] * b->dim[1] + y * b->dim[0]);
            for (uint64_t x = lo[0]; x < hi[0]; ++x) {
                const uint8_t* p = row + 4 * x;
                double d0 = (double)p[0] - av[0], d1 = (double)p[1] - av[1];
                double d2 = (double)p[2] - av[2], d3 = (double)p[3] - av[3];
                s += ((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3;
            }
        }
    *avg_out = avg;
    *split_out = sqrt(s / nd) > b->threshold;
}

/* detail::construct (OctreeConstruction.h:124-194) */
static uint32_t construct(Builder* b, const uint64_t off[3], uint64_t extent, uint64_t depth) {
    if (b->oom) return 0;
    if (depth > b->stats->depth) b->stats->depth = depth;
    Node node;
    memset(&node, 0, sizeof(node));
    int inside = off[0] < b->dim[0] && off[1] < b->dim[1] && off[2] < b->dim[2];
    if (!inside) {
        node.is_leaf_depth = LEAF | (uint32_t)depth;
        return insert(b, &node, 1);
    }
    /* the reference names this "partly_in_grid"; it means fully inside */
    int fully = off[0] + extent <= b->dim[0] && off[1] + extent <= b->dim[1] &&
                off[2] + extent <= b->dim[2];
    uint32_t avg;
    int split;
    grid_scan(b, off, extent, &avg, &split);
    if ((!split && fully) || extent == 1) {
        node.color = avg;
        node.is_leaf_depth = LEAF | (uint32_t)depth;
        return insert(b, &node, 1);
    }
    uint64_t h = extent / 2;
    int child = 0;
    node.color = avg;
    node.is_leaf_depth = (uint32_t)depth;
    for (int xi = 0; xi < 2; ++xi)
        for (int yi = 0; yi < 2; ++yi)
            for (int zi = 0; zi < 2; ++zi) {
                uint64_t co[3] = {off[0] + (xi ? h : 0), off[1] + (yi ? h : 0), off[2] + (zi ? h : 0)};
                node.children[child++] = construct(b, co, h, depth + 1);
            }
    return insert(b, &node, 0);
}

/* Octree::find (Octree.cpp:116-153): index of the node at depth <= max_depth
 * containing pos, or 0 when pos is outside (negative positions wrap). */
static uint64_t tree_find(const Node* nodes, uint64_t side, const uint64_t pos[3], uint64_t max_depth) {
    uint64_t extent = side;
    if (pos[0] >= extent || pos[1] >= extent || pos[2] >= extent) return 0;
    uint64_t index = 0, off[3] = {0, 0, 0};
    for (;;) {
        extent /= 2;
        if ((nodes[index].is_leaf_depth & LEAF) || extent == 0 || max_depth == 0) return index;
        uint32_t ci = 0;
        if (pos[0] >= off[0] + extent) { ci |= 4; off[0] += extent; }
        if (pos[1] >= off[1] + extent) { ci |= 2; off[1] += extent; }
        if (pos[2] >= off[2] + extent) { ci |= 1; off[2] += extent; }
        index = nodes[index].children[ci];
        --max_depth;
    }
}

/* Octree::walk_leaves_r + generate_ropes (Octree.cpp:155-201) */
static void ropes_r(Node* nodes, uint64_t side, uint64_t index, const uint64_t pos[3], uint64_t extent,
                    uint64_t depth) {
    Node* node = &nodes[index];
    if (node->is_leaf_depth & LEAF) {
        static const int64_t dirs[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        uint32_t r[6];
        for (int k = 0; k < 6; ++k) {
            uint64_t p[3];
            for (int a = 0; a < 3; ++a) p[a] = pos[a] + (uint64_t)(dirs[k][a] * (int64_t)extent);
            r[k] = (uint32_t)tree_find(nodes, side, p, depth);
        }
        for (int k = 0; k < 6; ++k) node->children[k] = r[k];
        return;
    }
    uint64_t h = extent / 2;
    int child = 0;
    for (int xi = 0; xi < 2; ++xi)
        for (int yi = 0; yi < 2; ++yi)
            for (int zi = 0; zi < 2; ++zi) {
                uint64_t cp[3] = {pos[0] + (xi ? h : 0), pos[1] + (yi ? h : 0), pos[2] + (zi ? h : 0)};
                ropes_r(nodes, side, nodes[index].children[child++], cp, h, depth + 1);
            }
}

static uint64_t ceil_pow2(uint64_t x) {
    --x;
    x |= x >> 1;
    x |= x >> 2;
    x |= x >> 4;
    x |= x >> 8;
    x |= x >> 16;
    x |= x >> 32;
    return ++x;
}

int xo_build_svo(const uint8_t* rgba, const uint32_t dim[3], int type, int heuristic, double threshold,
                 uint32_t** nodes_out, xo_build_stats* stats) {
    if (!rgba || !dim || !nodes_out || !stats) return -1;
    if (!dim[0] || !dim[1] || !dim[2]) return -1;
    if (type < XO_TYPE_SPARSE || type > XO_TYPE_ROPE) return -1;
    Builder b;
    memset(&b, 0, sizeof(b));
    memset(stats, 0, sizeof(*stats));
    b.rgba = rgba;
    for (int i = 0; i < 3; ++i) b.dim[i] = dim[i];
    b.heuristic = heuristic;
    b.threshold = threshold;
    b.dag = type == XO_TYPE_DAG;
    b.stats = stats;
    uint64_t side = ceil_pow2(dim[0]);
    if (ceil_pow2(dim[1]) > side) side = ceil_pow2(dim[1]);
    if (ceil_pow2(dim[2]) > side) side = ceil_pow2(dim[2]);
    uint64_t zero[3] = {0, 0, 0};
    construct(&b, zero, side, 0);
    free(b.cache.slots);
    if (b.oom) {
        free(b.nodes.v);
        return -2;
    }
    /* OctreeBuilder::build (OctreeConstruction.h:92-112) */
    Node* v = b.nodes.v;
    uint64_t n = b.nodes.n;
    for (uint64_t i = 0; i < n / 2; ++i) {
        Node t = v[i];
        v[i] = v[n - 1 - i];
        v[n - 1 - i] = t;
    }
    uint32_t end = (uint32_t)n - 1;
    for (uint64_t i = 0; i < n; ++i) {
        for (int k = 0; k < 8; ++k) v[i].children[k] = (v[i].is_leaf_depth & LEAF) ? 0 : end - v[i].children[k];
    }
    if (type == XO_TYPE_ROPE) ropes_r(v, side, 0, zero, side, 0);
    stats->side = side;
    stats->n_nodes = n;
    *nodes_out = (uint32_t*)v;
    return 0;
}

void xo_free(void* p) { free(p); }
