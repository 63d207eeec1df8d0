/*
 * mc_oracle.c -- CPU restatement of the reference kvs::MarchingCubes path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * implementation in kvs_gb300/csrc and the CPU baseline that bench.py times
 * when the reference itself is not built on the host.  Nothing in the
 * product links, loads or calls it.
 *
 * Parity of this restatement is pinned against the reference compiled from its
 * own sources (oracle/Makefile.ref + oracle/ref_driver.cpp) and against the
 * golden fixtures in tests/golden/ generated from that build.
 *
 * Every function cites the reference file:line it restates (paths relative
 * to the reference's Source/Core).  Build with -ffp-contract=off: the reference
 * arithmetic is the uncontracted IEEE sequence.
 *
 * The 256-case triangle table and the 12-edge endpoint table are the standard
 * marching-cubes tables that Visualization/Mapper/MarchingCubesTable.cpp:16-290
 * holds; they are read from kvs_gb300/csrc/mc_tables.h (the same data the
 * CUDA kernels use), which tests check entry-for-entry against the reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../kvs_gb300/csrc/mc_tables.h"

/* dtype codes: the order of the reference's type switch (MarchingCubes.cpp:115-124) */
enum { MCO_I8, MCO_I16, MCO_I32, MCO_I64, MCO_U8, MCO_U16, MCO_U32, MCO_U64, MCO_F32, MCO_F64, MCO_NTYPES };

typedef struct {
    int success;              /* exec() return: 1 = this, 0 = nullptr            */
    int extracted;            /* 0 when the Equal(min,max) early exit was taken */
    float* coords;  uint64_t ncoords;       /* floats */
    float* normals; uint64_t nnormals;      /* floats */
    uint32_t* connections; uint64_t nconnections;
    unsigned char color[3];
    double vmin, vmax;        /* volume min/max after the call                 */
    float min_obj[3], max_obj[3];
    double seconds;
} mco_output;

/* ---------------------------------------------------------------- helpers */

/* growable buffers standing in for the reference's std::vector push_back */
typedef struct { float* p; uint64_t n, cap; } fbuf;
typedef struct { uint32_t* p; uint64_t n, cap; } ubuf;

static int fbuf_push3(fbuf* b, float x, float y, float z)
{
    if (b->n + 3 > b->cap) {
        uint64_t cap = b->cap ? b->cap * 2 : 1024;
        float* p = (float*)realloc(b->p, cap * sizeof(float));
        if (!p) return -1;
        b->p = p; b->cap = cap;
    }
    b->p[b->n++] = x; b->p[b->n++] = y; b->p[b->n++] = z;
    return 0;
}

static int ubuf_push3(ubuf* b, uint32_t x, uint32_t y, uint32_t z)
{
    if (b->n + 3 > b->cap) {
        uint64_t cap = b->cap ? b->cap * 2 : 1024;
        uint32_t* p = (uint32_t*)realloc(b->p, cap * sizeof(uint32_t));
        if (!p) return -1;
        b->p = p; b->cap = cap;
    }
    b->p[b->n++] = x; b->p[b->n++] = y; b->p[b->n++] = z;
    return 0;
}

/* Utility/Math.h:129-132 */
static inline double clampd(double a, double lo, double hi) { return a <= lo ? lo : (a <= hi ? a : hi); }
/* Utility/Math.h:63-66 (keeps -0.0 and NaN as they are, unlike fabs) */
static inline double absd(double a) { return (a < 0) ? -a : a; }

typedef struct { float x, y, z; } vec3;

/* Matrix/Vector3.h:479-485 */
static inline vec3 cross3(vec3 a, vec3 b)
{
    vec3 r;
    r.x = a.y * b.z - a.z * b.y;
    r.y = a.z * b.x - a.x * b.z;
    r.z = a.x * b.y - a.y * b.x;
    return r;
}
static inline vec3 sub3(vec3 a, vec3 b) { vec3 r = { a.x - b.x, a.y - b.y, a.z - b.z }; return r; }

/* ------------------------------------------------- per-dtype value access */

#define MCO_TYPE_LIST(X) \
    X(MCO_I8, int8_t) X(MCO_I16, int16_t) X(MCO_I32, int32_t) X(MCO_I64, int64_t) \
    X(MCO_U8, uint8_t) X(MCO_U16, uint16_t) X(MCO_U32, uint32_t) X(MCO_U64, uint64_t) \
    X(MCO_F32, float) X(MCO_F64, double)

/* Shared extraction state (MarchingCubes.cpp:156-173, 366-386). */
typedef struct {
    const void* values;
    int dtype;
    uint32_t nx, ny, nz;
    uint32_t line, slice;     /* numberOfNodesPerLine / PerSlice as UInt32 */
    double iso, vmin, vmax;
    vec3 min_coord, scale;
    uint32_t z0, z1;          /* cell planes visited by the duplicated loop */
} mc_state;

/*
 * Where the duplicated loop's triangles go: appended to coords/normals as the
 * reference's push_back does, or (chunk_tris > 0) folded into position-keyed
 * checksums per chunk of chunk_tris triangles, the same sums as
 * kvsmc_checksum_words over the coords (9 words per triangle) and normals
 * (3 words per triangle) arrays, so outputs too large to copy can be compared.
 */
typedef struct {
    fbuf* coords;
    fbuf* normals;
    uint64_t chunk_tris;
    uint64_t* coord_sums;
    uint64_t* normal_sums;
    uint64_t nchunks;
    uint64_t ntri;
    int overflow;             /* more triangles than nchunks * chunk_tris */
} mco_sink;

/* the checksum term of word w at index i (kvsmc_checksum_words) */
static inline uint64_t mco_mix(uint64_t i, uint32_t w)
{
    uint64_t x = (i * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)w * 0xC2B2AE3D27D4EB4Full);
    x ^= x >> 31;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 29;
    return x;
}

static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static int sink_triangle(mco_sink* k, const vec3 q[3], vec3 n)
{
    if (!k->chunk_tris) {
        for (int j = 0; j < 3; ++j)
            if (fbuf_push3(k->coords, q[j].x, q[j].y, q[j].z)) return -1;
        if (fbuf_push3(k->normals, n.x, n.y, n.z)) return -1;
    } else {
        const uint64_t t = k->ntri, c = t / k->chunk_tris;
        if (c >= k->nchunks) {
            k->overflow = 1;
        } else {
            const float w[9] = { q[0].x, q[0].y, q[0].z, q[1].x, q[1].y, q[1].z, q[2].x, q[2].y, q[2].z };
            uint64_t h = 0;
            for (int j = 0; j < 9; ++j) h += mco_mix(9 * t + (uint64_t)j, fbits(w[j]));
            k->coord_sums[c] += h;
            k->normal_sums[c] += mco_mix(3 * t, fbits(n.x)) + mco_mix(3 * t + 1, fbits(n.y)) +
                                 mco_mix(3 * t + 2, fbits(n.z));
        }
    }
    k->ntri++;
    return 0;
}

/*
 * GetMinMaxValues<T>, veclen == 1 (Visualization/Object/StructuredVolumeObject.cpp:66-85):
 * sequential Min/Max starting from the first value; Math::Min(a,b) = a<b?a:b.
 */
#define MCO_MINMAX(CODE, T) \
    static void minmax_##CODE(const T* v, uint64_t n, double* mn, double* mx) { \
        T lo = v[0], hi = v[0]; \
        for (uint64_t i = 0; i < n; ++i) { \
            lo = (v[i] < lo) ? v[i] : lo; \
            hi = (v[i] > hi) ? v[i] : hi; \
        } \
        *mn = (double)lo; *mx = (double)hi; \
    }
MCO_TYPE_LIST(MCO_MINMAX)

int mco_minmax(int dtype, const void* values, uint64_t n, double* mn, double* mx)
{
    if (n == 0) return -1;
    switch (dtype) {
#define MCO_MM_CASE(CODE, T) case CODE: minmax_##CODE((const T*)values, n, mn, mx); return 0;
        MCO_TYPE_LIST(MCO_MM_CASE)
    }
    return -1;
}

/*
 * interpolate_vertex<T> (MarchingCubes.cpp:327-356) followed by the
 * (p + min_coord) * scale_factor lambda (MarchingCubes.cpp:168-173).
 * Endpoint index computed in double (:342-343); values clamped to the volume's
 * [min,max] (:347-348); ratio = Abs((iso-v0)/(v1-v0)) (:349); each axis
 * (1.0 - ratio)*a + ratio*b in double, rounded to float (:351-355).
 */
#define MCO_INTERP(CODE, T) \
    static vec3 interp_##CODE(const mc_state* s, vec3 a, vec3 b) { \
        const T* vals = (const T*)s->values; \
        const double x0 = a.x, y0 = a.y, z0 = a.z, x1 = b.x, y1 = b.y, z1 = b.z; \
        const size_t i0 = (size_t)(x0 + y0 * (double)s->line + z0 * (double)s->slice); \
        const size_t i1 = (size_t)(x1 + y1 * (double)s->line + z1 * (double)s->slice); \
        double v0 = (double)vals[i0], v1 = (double)vals[i1]; \
        v0 = clampd(v0, s->vmin, s->vmax); \
        v1 = clampd(v1, s->vmin, s->vmax); \
        const double r = absd((s->iso - v0) / (v1 - v0)); \
        const double px = (1.0 - r) * x0 + r * x1; \
        const double py = (1.0 - r) * y0 + r * y1; \
        const double pz = (1.0 - r) * z0 + r * z1; \
        vec3 p = { (float)px, (float)py, (float)pz }; \
        vec3 q = { (p.x + s->min_coord.x) * s->scale.x, (p.y + s->min_coord.y) * s->scale.y, \
                   (p.z + s->min_coord.z) * s->scale.z }; \
        return q; \
    }
MCO_TYPE_LIST(MCO_INTERP)

/* calculate_table_index<T> (MarchingCubes.cpp:300-316): bit k set iff double(v_k) > iso */
#define MCO_CASE(CODE, T) \
    static inline unsigned case_##CODE(const T* v, const size_t* li, double iso) { \
        unsigned c = 0; \
        for (int k = 0; k < 8; ++k) if ((double)v[li[k]] > iso) c |= 1u << k; \
        return c; \
    }
MCO_TYPE_LIST(MCO_CASE)

/* corner node offsets in the order of MarchingCubes.cpp:187-194 */
static void cell_nodes(size_t base, uint32_t line, uint32_t slice, size_t li[8])
{
    li[0] = base;
    li[1] = base + 1;
    li[2] = base + 1 + line;
    li[3] = base + line;
    li[4] = base + slice;
    li[5] = base + 1 + slice;
    li[6] = base + 1 + line + slice;
    li[7] = base + line + slice;
}

/*
 * extract_surfaces_with_duplication<T> (MarchingCubes.cpp:156-243):
 * cells z, y, x (x fastest); per triangle the edges (e[i], e[i+2], e[i+1]);
 * each edge interpolated in the table's direction; normal (v23-v01)x(v45-v01).
 */
#define MCO_DUP(CODE, T) \
    static int dup_##CODE(const mc_state* s, mco_sink* sink) { \
        const T* vals = (const T*)s->values; \
        const uint32_t cx = s->nx - 1, cy = s->ny - 1; \
        size_t li[8]; \
        for (uint32_t z = s->z0; z < s->z1; ++z) \
        for (uint32_t y = 0; y < cy; ++y) \
        for (uint32_t x = 0; x < cx; ++x) { \
            const size_t base = (size_t)x + (size_t)y * s->line + (size_t)z * s->slice; \
            cell_nodes(base, s->line, s->slice, li); \
            const unsigned c = case_##CODE(vals, li, s->iso); \
            if (c == 0 || c == 255) continue; \
            const signed char* tri = MC_TRIANGLE_TABLE[c]; \
            for (int i = 0; tri[i] != -1; i += 3) { \
                const int e[3] = { tri[i], tri[i + 2], tri[i + 1] }; \
                vec3 q[3]; \
                for (int k = 0; k < 3; ++k) { \
                    const signed char* a = MC_EDGE_VERTEX[e[k]][0]; \
                    const signed char* b = MC_EDGE_VERTEX[e[k]][1]; \
                    vec3 pa = { (float)(x + (uint32_t)a[0]), (float)(y + (uint32_t)a[1]), (float)(z + (uint32_t)a[2]) }; \
                    vec3 pb = { (float)(x + (uint32_t)b[0]), (float)(y + (uint32_t)b[1]), (float)(z + (uint32_t)b[2]) }; \
                    q[k] = interp_##CODE(s, pa, pb); \
                } \
                const vec3 n = cross3(sub3(q[1], q[0]), sub3(q[2], q[0])); \
                if (sink_triangle(sink, q, n)) return -1; \
            } \
        } \
        return 0; \
    }
MCO_TYPE_LIST(MCO_DUP)

/*
 * calculate_isopoints<T> (MarchingCubes.cpp:366-446): every node in z, y, x
 * order; its x-, y- then z-edge (when inside the grid) gets a vertex if the
 * endpoints classify differently, interpolated from this (lower) node; ids
 * are a running UInt32 counter stored in a 3-per-node map.
 */
#define MCO_ISOPOINTS(CODE, T) \
    static int isopoints_##CODE(const mc_state* s, uint32_t* vmap, fbuf* coords) { \
        const T* vals = (const T*)s->values; \
        const uint32_t cx = s->nx - 1, cy = s->ny - 1, cz = s->nz - 1; \
        uint32_t nv = 0; \
        for (uint32_t z = 0; z < s->nz; ++z) \
        for (uint32_t y = 0; y < s->ny; ++y) \
        for (uint32_t x = 0; x < s->nx; ++x) { \
            const size_t id0 = (size_t)x + (size_t)y * s->line + (size_t)z * s->slice; \
            const int b0 = (double)vals[id0] > s->iso; \
            const vec3 p = { (float)x, (float)y, (float)z }; \
            if (x != cx && ((double)vals[id0 + 1] > s->iso) != b0) { \
                vec3 pb = { (float)(x + 1), (float)y, (float)z }; \
                vec3 q = interp_##CODE(s, p, pb); \
                if (fbuf_push3(coords, q.x, q.y, q.z)) return -1; \
                vmap[3 * id0] = nv++; \
            } \
            if (y != cy && ((double)vals[id0 + s->line] > s->iso) != b0) { \
                vec3 pb = { (float)x, (float)(y + 1), (float)z }; \
                vec3 q = interp_##CODE(s, p, pb); \
                if (fbuf_push3(coords, q.x, q.y, q.z)) return -1; \
                vmap[3 * id0 + 1] = nv++; \
            } \
            if (z != cz && ((double)vals[id0 + s->slice] > s->iso) != b0) { \
                vec3 pb = { (float)x, (float)y, (float)(z + 1) }; \
                vec3 q = interp_##CODE(s, p, pb); \
                if (fbuf_push3(coords, q.x, q.y, q.z)) return -1; \
                vmap[3 * id0 + 2] = nv++; \
            } \
        } \
        return 0; \
    }
MCO_TYPE_LIST(MCO_ISOPOINTS)

/*
 * connect_isopoints<T> (MarchingCubes.cpp:456-521): cells in z, y, x order;
 * the cell's 12 edges mapped to (node, axis) slots of the vertex map
 * (:493-504); per triangle (e[i], e[i+2], e[i+1]).  The reference narrows the
 * slot index to int (:508-510), which is exact while 3 * nodes < 2^31.
 */
#define MCO_CONNECT(CODE, T) \
    static int connect_##CODE(const mc_state* s, const uint32_t* vmap, ubuf* conn) { \
        const T* vals = (const T*)s->values; \
        const uint32_t cx = s->nx - 1, cy = s->ny - 1, cz = s->nz - 1; \
        size_t li[8], le[12]; \
        for (uint32_t z = 0; z < cz; ++z) \
        for (uint32_t y = 0; y < cy; ++y) \
        for (uint32_t x = 0; x < cx; ++x) { \
            const size_t base = (size_t)x + (size_t)y * s->line + (size_t)z * s->slice; \
            cell_nodes(base, s->line, s->slice, li); \
            const unsigned c = case_##CODE(vals, li, s->iso); \
            if (c == 0 || c == 255) continue; \
            const size_t e0 = 3 * base; \
            le[0] = e0;                          /* x-edge of node 0 */ \
            le[1] = e0 + 3 + 1;                  /* y-edge of node 1 */ \
            le[2] = e0 + 3 * (size_t)s->line;    /* x-edge of node 3 */ \
            le[3] = e0 + 1;                      /* y-edge of node 0 */ \
            le[4] = le[0] + 3 * (size_t)s->slice; \
            le[5] = le[1] + 3 * (size_t)s->slice; \
            le[6] = le[2] + 3 * (size_t)s->slice; \
            le[7] = le[3] + 3 * (size_t)s->slice; \
            le[8] = e0 + 2;                      /* z-edge of node 0 */ \
            le[9] = le[8] + 3;                   /* z-edge of node 1 */ \
            le[10] = le[8] + 3 + 3 * (size_t)s->line; /* z-edge of node 2 */ \
            le[11] = le[8] + 3 * (size_t)s->line;     /* z-edge of node 3 */ \
            const signed char* tri = MC_TRIANGLE_TABLE[c]; \
            for (int i = 0; tri[i] != -1; i += 3) { \
                if (ubuf_push3(conn, vmap[le[tri[i]]], vmap[le[tri[i + 2]]], vmap[le[tri[i + 1]]])) return -1; \
            } \
        } \
        return 0; \
    }
MCO_TYPE_LIST(MCO_CONNECT)

/* calculate_normals_on_polygon (MarchingCubes.cpp:531-560) */
static float* normals_on_polygon(const fbuf* coords, const ubuf* conn)
{
    if (coords->n == 0) return NULL;
    float* nrm = (float*)calloc(conn->n ? conn->n : 1, sizeof(float));
    for (uint64_t i = 0; i < conn->n; i += 3) {
        const float* a = coords->p + 3 * (uint64_t)conn->p[i];
        const float* b = coords->p + 3 * (uint64_t)conn->p[i + 1];
        const float* c = coords->p + 3 * (uint64_t)conn->p[i + 2];
        vec3 v0 = { a[0], a[1], a[2] }, v1 = { b[0], b[1], b[2] }, v2 = { c[0], c[1], c[2] };
        vec3 n = cross3(sub3(v1, v0), sub3(v2, v0));
        nrm[i] = n.x; nrm[i + 1] = n.y; nrm[i + 2] = n.z;
    }
    return nrm;
}

/* calculate_normals_on_vertex (MarchingCubes.cpp:569-605): += in triangle order from 0.0f */
static float* normals_on_vertex(const fbuf* coords, const ubuf* conn)
{
    if (coords->n == 0) return NULL;
    float* nrm = (float*)calloc(coords->n, sizeof(float));
    for (uint64_t i = 0; i < conn->n; i += 3) {
        const uint64_t i0 = 3 * (uint64_t)conn->p[i], i1 = 3 * (uint64_t)conn->p[i + 1],
                       i2 = 3 * (uint64_t)conn->p[i + 2];
        vec3 v0 = { coords->p[i0], coords->p[i0 + 1], coords->p[i0 + 2] };
        vec3 v1 = { coords->p[i1], coords->p[i1 + 1], coords->p[i1 + 2] };
        vec3 v2 = { coords->p[i2], coords->p[i2 + 1], coords->p[i2 + 2] };
        vec3 n = cross3(sub3(v1, v0), sub3(v2, v0));
        nrm[i0] += n.x; nrm[i0 + 1] += n.y; nrm[i0 + 2] += n.z;
        nrm[i1] += n.x; nrm[i1 + 1] += n.y; nrm[i1 + 2] += n.z;
        nrm[i2] += n.x; nrm[i2 + 1] += n.y; nrm[i2 + 2] += n.z;
    }
    return nrm;
}

/*
 * The extraction body for one (volume, isolevel) once min/max, bbox and
 * scale are known: extract_surfaces<T> (MarchingCubes.cpp:141-147).
 * mode: 0 = duplicated + polygon normals, 1 = shared vertices + polygon
 * normals, 2 = shared vertices + vertex normals.
 * Returns 0, or -1 on allocation failure.
 */
int mco_extract(int dtype, const void* values, uint32_t nx, uint32_t ny, uint32_t nz,
                double iso, int mode, double vmin, double vmax,
                const float min_coord[3], const float scale[3], mco_output* out)
{
    mc_state s;
    s.values = values; s.dtype = dtype; s.nx = nx; s.ny = ny; s.nz = nz;
    s.line = nx; s.slice = nx * ny;
    s.iso = iso; s.vmin = vmin; s.vmax = vmax;
    s.min_coord.x = min_coord[0]; s.min_coord.y = min_coord[1]; s.min_coord.z = min_coord[2];
    s.scale.x = scale[0]; s.scale.y = scale[1]; s.scale.z = scale[2];
    s.z0 = 0; s.z1 = nz - 1;

    fbuf coords = { 0 }, normals = { 0 };
    ubuf conn = { 0 };
    int rc = 0;
    if (mode == 0) {
        mco_sink sink;
        memset(&sink, 0, sizeof sink);
        sink.coords = &coords;
        sink.normals = &normals;
        switch (dtype) {
#define MCO_DUP_CASE(CODE, T) case CODE: rc = dup_##CODE(&s, &sink); break;
            MCO_TYPE_LIST(MCO_DUP_CASE)
        default: return -2;
        }
    } else {
        /* extract_surfaces_without_duplication<T> (MarchingCubes.cpp:252-290) */
        const uint64_t nnodes = (uint64_t)nx * ny * nz;
        uint32_t* vmap = (uint32_t*)calloc(3 * nnodes, sizeof(uint32_t));
        if (!vmap) return -1;
        switch (dtype) {
#define MCO_ND_CASE(CODE, T) case CODE: rc = isopoints_##CODE(&s, vmap, &coords); \
            if (!rc) rc = connect_##CODE(&s, vmap, &conn); break;
            MCO_TYPE_LIST(MCO_ND_CASE)
        default: free(vmap); return -2;
        }
        free(vmap);
        if (!rc) {
            float* n = (mode == 1) ? normals_on_polygon(&coords, &conn) : normals_on_vertex(&coords, &conn);
            normals.p = n;
            normals.n = n ? ((mode == 1) ? conn.n : coords.n) : 0;
        }
    }
    if (rc) { free(coords.p); free(normals.p); free(conn.p); return -1; }
    out->coords = coords.p; out->ncoords = coords.n;
    out->normals = normals.p; out->nnormals = normals.n;
    out->connections = conn.p; out->nconnections = conn.n;
    return 0;
}

/*
 * The duplicated loop of mco_extract (extract_surfaces_with_duplication<T>,
 * MarchingCubes.cpp:156-243) over the cell planes [z0, z1) of the whole
 * volume, with the triangles folded into per-chunk checksums instead of
 * stored (see mco_sink); coordinates are the volume's own, so a slab's
 * triangles are the same bits as that stretch of a whole-volume run.
 * Returns 0, -2 for a bad dtype or range, -3 when the triangles overflow
 * nchunks * chunk_tris (*ntri is still the count).
 */
int mco_dup_checksum(int dtype, const void* values, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t z0,
                     uint32_t z1, double iso, double vmin, double vmax, const float min_coord[3],
                     const float scale[3], uint64_t chunk_tris, uint64_t* coord_sums, uint64_t* normal_sums,
                     uint64_t nchunks, uint64_t* ntri)
{
    if (nx < 2 || ny < 2 || nz < 2 || z0 > z1 || z1 > nz - 1 || chunk_tris == 0) return -2;
    mc_state s;
    s.values = values; s.dtype = dtype; s.nx = nx; s.ny = ny; s.nz = nz;
    s.line = nx; s.slice = nx * ny;
    s.iso = iso; s.vmin = vmin; s.vmax = vmax;
    s.min_coord.x = min_coord[0]; s.min_coord.y = min_coord[1]; s.min_coord.z = min_coord[2];
    s.scale.x = scale[0]; s.scale.y = scale[1]; s.scale.z = scale[2];
    s.z0 = z0; s.z1 = z1;
    mco_sink sink;
    memset(&sink, 0, sizeof sink);
    sink.chunk_tris = chunk_tris;
    sink.coord_sums = coord_sums;
    sink.normal_sums = normal_sums;
    sink.nchunks = nchunks;
    memset(coord_sums, 0, nchunks * sizeof(uint64_t));
    memset(normal_sums, 0, nchunks * sizeof(uint64_t));
    int rc = 0;
    switch (dtype) {
#define MCO_DUP_SUM_CASE(CODE, T) case CODE: rc = dup_##CODE(&s, &sink); break;
        MCO_TYPE_LIST(MCO_DUP_SUM_CASE)
    default: return -2;
    }
    *ntri = sink.ntri;
    if (rc) return rc;
    return sink.overflow ? -3 : 0;
}

/*
 * ColorMap::at (Visualization/Mapper/ColorMap.cpp:1043-1054) with
 * RGBColor::Mix (Image/RGBColor.cpp:23-31), Math::Mix (Utility/Math.h) and
 * RGBColor = Vec3 (Image/RGBColor.cpp:125-134).  table: resolution x RGB.
 */
void mco_color_at(const unsigned char* table, int resolution, float tf_min, float tf_max,
                  float value, unsigned char rgb[3])
{
    const float v0 = value <= tf_min ? tf_min : (value <= tf_max ? value : tf_max);
    const float r = (float)(resolution - 1);
    const float v = (v0 - tf_min) / (tf_max - tf_min) * r;
    const size_t s0 = (size_t)v;
    const size_t s1 = (s0 + 1 < (size_t)(resolution - 1)) ? s0 + 1 : (size_t)(resolution - 1);
    const float t = v - (float)s0;
    for (int k = 0; k < 3; ++k) {
        const float a = (float)table[3 * s0 + k] / 255.0f;
        const float b = (float)table[3 * s1 + k] / 255.0f;
        float m = a * (1 - t) + b * t;
        m = m <= 0.0f ? 0.0f : (m <= 1.0f ? m : 1.0f);
        const float f = m * 255.0f;
        rgb[k] = (unsigned char)(f >= 0 ? (int)(f + 0.5) : -(int)(0.5 - f));
    }
}

/*
 * The whole constructor -> exec -> mapping flow (MarchingCubes.cpp:25-132) for a
 * uniform or rectilinear structured volume with veclen 1:
 *   setRange (MapperBase.cpp:54-83): scan min/max unless preset; TF range
 *     [0,255] for u8, [-128,127] for i8, else float(min), float(max) (+1 when
 *     Equal), unless the TF already has a range;
 *   setMinMaxCoords (MapperBase.cpp:92-122, StructuredVolumeObject.cpp:348-386):
 *     uniform -> [0, res-1], rectilinear -> first/last coord per axis, unless preset;
 *   Equal(min,max) (Utility/Math.h:135-138, |a-b| < 1e-6) -> success, no output;
 *   VertexNormal forces shared vertices (MarchingCubes.cpp:70-73);
 *   scale = (max_coord - min_coord) / ncells in float (MarchingCubes.cpp:166-168).
 * grid_type: 0 uniform, 1 rectilinear (rect = nx+ny+nz floats).
 * normal_type: 0 vertex, 1 polygon (PolygonObject.h:50-55 numbering).
 */
int mco_marching_cubes(int dtype, const void* values, uint32_t nx, uint32_t ny, uint32_t nz,
                       double iso, int normal_type, int duplication,
                       int has_minmax, double vmin, double vmax,
                       int grid_type, const float* rect,
                       int has_obj, const float* min_obj, const float* max_obj,
                       const unsigned char* cmap, int cmap_res, int tf_has_range, float tf_min, float tf_max,
                       mco_output* out)
{
    memset(out, 0, sizeof(*out));
    const uint64_t n = (uint64_t)nx * ny * nz;
    if (n == 0 || dtype < 0 || dtype >= MCO_NTYPES) return -2;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);

    if (!has_minmax) mco_minmax(dtype, values, n, &vmin, &vmax);
    out->vmin = vmin; out->vmax = vmax;

    if (!tf_has_range) {
        if (dtype == MCO_I8) { tf_min = -128; tf_max = 127; }
        else if (dtype == MCO_U8) { tf_min = 0; tf_max = 255; }
        else {
            tf_min = (float)vmin; tf_max = (float)vmax;
            if (fabsf(tf_min - tf_max) < 1.e-6) tf_max = tf_max + 1.0f;
        }
    }

    float mn[3], mx[3];
    if (has_obj) { memcpy(mn, min_obj, sizeof mn); memcpy(mx, max_obj, sizeof mx); }
    else if (grid_type == 1) {
        mn[0] = rect[0]; mn[1] = rect[nx]; mn[2] = rect[nx + ny];
        mx[0] = rect[nx - 1]; mx[1] = rect[nx + ny - 1]; mx[2] = rect[nx + ny + nz - 1];
    } else {
        mn[0] = mn[1] = mn[2] = 0.0f;
        mx[0] = (float)nx - 1.0f; mx[1] = (float)ny - 1.0f; mx[2] = (float)nz - 1.0f;
    }
    memcpy(out->min_obj, mn, sizeof mn); memcpy(out->max_obj, mx, sizeof mx);
    out->success = 1;

    if (absd(vmin - vmax) < 1.e-6) { out->extracted = 0; goto done; }
    out->extracted = 1;

    {
        const float scale[3] = { (mx[0] - mn[0]) / (float)(nx - 1), (mx[1] - mn[1]) / (float)(ny - 1),
                                 (mx[2] - mn[2]) / (float)(nz - 1) };
        const int mode = (normal_type == 0) ? 2 : (duplication ? 0 : 1);
        const int rc = mco_extract(dtype, values, nx, ny, nz, iso, mode, vmin, vmax, mn, scale, out);
        if (rc) return rc;
    }
    if (cmap && out->ncoords > 0) mco_color_at(cmap, cmap_res, tf_min, tf_max, (float)iso, out->color);
done:
    clock_gettime(CLOCK_MONOTONIC, &t1);
    out->seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    return 0;
}

void mco_free(mco_output* o)
{
    free(o->coords); free(o->normals); free(o->connections);
    memset(o, 0, sizeof(*o));
}
