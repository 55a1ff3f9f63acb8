/* A CPU model of the two traversals in aurora_gb300/csrc/aur_traverse.cuh:
 * `traverse` (one ray per lane: depth first, near child first, range trail,
 * subtree-box pruning) and `traverse_packet` (a warp of 32 rays of one
 * direction octant walking one node sequence, each lane with its own range,
 * best hit and pending far children), both restated step by step with the
 * same float operations, plus the reference's own walk (intersect() /
 * intersectAny(), kernels/lib/intersect.cuh:36-152: an explicit stack, no
 * pruning). For every ray it checks that all three give the same closest hit
 * (index and the bits of t, u, v) and the same any-hit occluder.
 *
 * Input files (little-endian): the NMH-ordered soup (count x 9 floats,
 * [x1 x2 x3 y1 y2 y3 z1 z2 z3]), perm (count u32), rays (n x 8 floats: origin,
 * tmax, direction, pad; n a multiple of 32, each chunk of 32 of one octant).
 * Usage: packet_model soup perm rays count n -> prints "<rays> <mismatches>". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define EPS 1e-7f
#define INF 1e6f
#define NOPRIM 0xFFFFFFFFu
#define SKIP 0x80000000u

typedef struct { float x, y, z; } f3;
static float sel(uint32_t a, f3 v) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
static uint32_t bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static uint32_t count, nodes;
static const float* V;
static const uint32_t* perm;
static float* box;   /* per node: padded subtree box of the node (lo xyz, hi xyz) */

/* ray.cuh:198-223, Moller-Trumbore with culling, no fused operations */
static int tri(f3 p, f3 d, uint32_t i, float* u, float* v, float* t) {
    const float* q = V + (size_t)i * 9;
    const f3 v1 = {q[0], q[3], q[6]};
    const f3 e1 = {q[1] - q[0], q[4] - q[3], q[7] - q[6]};
    const f3 e2 = {q[2] - q[0], q[5] - q[3], q[8] - q[6]};
    const f3 P = {d.y * e2.z - d.z * e2.y, d.z * e2.x - d.x * e2.z, d.x * e2.y - d.y * e2.x};
    const float det = e1.x * P.x + e1.y * P.y + e1.z * P.z;
    if (det < EPS) return 0;
    const float inv = 1.0f / det;
    const f3 T = {p.x - v1.x, p.y - v1.y, p.z - v1.z};
    *u = (T.x * P.x + T.y * P.y + T.z * P.z) * inv;
    if (*u < 0.0f || *u > 1.0f) return 0;
    const f3 Q = {T.y * e1.z - T.z * e1.y, T.z * e1.x - T.x * e1.z, T.x * e1.y - T.y * e1.x};
    *v = (d.x * Q.x + d.y * Q.y + d.z * Q.z) * inv;
    if (*v < 0.0f || *u + *v > 1.0f) return 0;
    *t = (e2.x * Q.x + e2.y * Q.y + e2.z * Q.z) * inv;
    return 1;
}

static void slab(uint32_t k, uint32_t a, float* lo, float* hi) {
    float l = INFINITY, h = -INFINITY;
    for (int t = 0; t < 2; ++t)
        for (int c = 0; c < 3; ++c) {
            const float x = V[(size_t)(2 * k + t) * 9 + 3 * a + c];
            l = fminf(l, x);
            h = fmaxf(h, x);
        }
    *lo = l;
    *hi = h;
}

/* ray.cuh:225-237 with the cumulative range */
static int slab_test(uint32_t k, uint32_t a, f3 p, f3 d, float lo, float hi, float best, float* nlo, float* nhi) {
    float s0, s1;
    slab(k, a, &s0, &s1);
    const float d0 = (s0 - sel(a, p)) / sel(a, d), d1 = (s1 - sel(a, p)) / sel(a, d);
    *nlo = fmaxf(fminf(d0, d1), lo);
    *nhi = fminf(fmaxf(d0, d1), hi);
    return *nlo <= *nhi && *nlo <= best;
}

/* the tests of a node's two triangles; returns 1 on an any-hit */
static int node_tris(int any, uint32_t k, f3 p, f3 d, float* best_t, float* bu, float* bv, uint32_t* best) {
    for (uint32_t j = 0; j < 2; ++j) {
        const uint32_t idx = 2 * k + j;
        float u, v, t;
        if (!tri(p, d, idx, &u, &v, &t) || !(t > EPS)) continue;
        if (any) {
            if (t < *best_t) { *best = idx; return 1; }
        } else if (t < *best_t || (t == *best_t && *best != NOPRIM && perm[idx] < perm[*best])) {
            *best_t = t; *bu = u; *bv = v; *best = idx;
        }
    }
    return 0;
}

static f3 box_inv(f3 d) {
    f3 r = {1.0f / copysignf(fmaxf(fabsf(d.x), 1e-30f), d.x), 1.0f / copysignf(fmaxf(fabsf(d.y), 1e-30f), d.y),
            1.0f / copysignf(fmaxf(fabsf(d.z), 1e-30f), d.z)};
    return r;
}

static int box_hit(uint32_t c, f3 poi, f3 inv, float tl) {
    const float* b = box + 6 * (size_t)c;
    const float x0 = fmaf(b[0], inv.x, -poi.x), x1 = fmaf(b[3], inv.x, -poi.x);
    const float y0 = fmaf(b[1], inv.y, -poi.y), y1 = fmaf(b[4], inv.y, -poi.y);
    const float z0 = fmaf(b[2], inv.z, -poi.z), z1 = fmaf(b[5], inv.z, -poi.z);
    const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), 0.0f));
    const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tl));
    return tn * 0.9999f <= tf * 1.0001f;
}

typedef struct { uint32_t best; float t, u, v; } Hit;

/* the reference's walk: explicit stack of (index, axis, range), no pruning */
static Hit reference(int any, f3 p, f3 d, float tmax) {
    struct { uint32_t k, a; float lo, hi; } st[128];
    int sp = 0;
    Hit h = {NOPRIM, tmax, 0.0f, 0.0f};
    st[sp].k = 0; st[sp].a = 0; st[sp].lo = EPS; st[sp].hi = INF; ++sp;
    while (sp > 0) {
        --sp;
        const uint32_t k = st[sp].k, a = st[sp].a;
        if (k >= nodes) continue;
        float nlo, nhi;
        if (!slab_test(k, a, p, d, st[sp].lo, st[sp].hi, h.t, &nlo, &nhi)) continue;
        if (node_tris(any, k, p, d, &h.t, &h.u, &h.v, &h.best)) return h;
        const uint32_t na = (a + 1) % 3;
        uint32_t n = 2 * k + 1, f = 2 * k + 2;
        if (sel(na, d) < 0.0f) { n = 2 * k + 2; f = 2 * k + 1; }
        st[sp].k = f; st[sp].a = na; st[sp].lo = nlo; st[sp].hi = nhi; ++sp;
        st[sp].k = n; st[sp].a = na; st[sp].lo = nlo; st[sp].hi = nhi; ++sp;
    }
    return h;
}

/* traverse(): range trail, far children by heap position, box pruning */
static Hit per_lane(int any, f3 p, f3 d, float tmax) {
    float slo[40], shi[40];
    const f3 inv = box_inv(d);
    Hit h = {NOPRIM, tmax, 0.0f, 0.0f};
    uint32_t k = 0, lvl = 0, a = 0, trail = 0;
    float lo = EPS, hi = INF;
    for (;;) {
        float nlo = 0, nhi = 0;
        int crossed = 0;
        while (!crossed) {
            if (k < nodes && slab_test(k, a, p, d, lo, hi, h.t, &nlo, &nhi)) { crossed = 1; break; }
            if (trail == 0) return h;
            const uint32_t L = 31u - (uint32_t)__builtin_clz(trail);
            trail &= ~(1u << L);
            k = ((((k & ~SKIP) + 1u) >> (lvl - L)) ^ 1u) - 1u;
            lvl = L; a = L % 3u; lo = slo[L]; hi = shi[L];
        }
        if (node_tris(any, k, p, d, &h.t, &h.u, &h.v, &h.best)) return h;
        const uint32_t na = a == 2 ? 0 : a + 1;
        const int neg = sel(na, d) < 0.0f;
        const uint32_t c1 = 2 * k + 1;
        int h1 = c1 < nodes, h2 = c1 + 1 < nodes;
        if (h1) {
            const f3 poi = {p.x * inv.x, p.y * inv.y, p.z * inv.z};
            h1 = box_hit(c1, poi, inv, h.t);
            if (h2) h2 = box_hit(c1 + 1, poi, inv, h.t);
        }
        const int near_ok = neg ? h2 : h1, far_ok = neg ? h1 : h2;
        const uint32_t L = lvl + 1;
        if (far_ok) { slo[L] = nlo; shi[L] = nhi; trail |= 1u << L; }
        k = (neg ? c1 + 1 : c1) | (near_ok ? 0u : SKIP);
        lvl = L; a = na; lo = nlo; hi = nhi;
    }
}

/* traverse_packet(): the warp's node sequence, per-lane decisions */
static void packet(int any, const f3* p, const f3* d, const float* tmax, uint32_t oct, Hit* out) {
    float slo[32][40], shi[32][40], lo[32], hi[32], nlo[32], nhi[32];
    uint32_t trail[32];
    int act[32], crossed[32];
    f3 inv[32];
    for (int l = 0; l < 32; ++l) {
        inv[l] = box_inv(d[l]);
        out[l].best = NOPRIM; out[l].t = tmax[l]; out[l].u = out[l].v = 0.0f;
        trail[l] = 0; act[l] = 1; lo[l] = EPS; hi[l] = INF;
    }
    uint32_t k = 0, lvl = 0, ax = 0;
    for (;;) {
        int any_act = 0;
        for (int l = 0; l < 32; ++l) any_act |= act[l];
        if (any_act && k < nodes) {
            int any_crossed = 0;
            for (int l = 0; l < 32; ++l) {
                crossed[l] = act[l] && slab_test(k, ax, p[l], d[l], lo[l], hi[l], out[l].t, &nlo[l], &nhi[l]);
                if (crossed[l] && node_tris(any, k, p[l], d[l], &out[l].t, &out[l].u, &out[l].v, &out[l].best)) {
                    crossed[l] = 0;
                    trail[l] = 0;
                }
                any_crossed |= crossed[l];
            }
            const uint32_t c1 = 2 * k + 1;
            if (any_crossed && c1 < nodes) {
                const uint32_t na = ax == 2 ? 0 : ax + 1;
                const int neg = (oct >> na) & 1u;
                const uint32_t L = lvl + 1;
                int any_near = 0;
                for (int l = 0; l < 32; ++l) {
                    int h1 = 0, h2 = 0;
                    if (crossed[l]) {
                        const f3 poi = {p[l].x * inv[l].x, p[l].y * inv[l].y, p[l].z * inv[l].z};
                        h1 = box_hit(c1, poi, inv[l], out[l].t);
                        if (c1 + 1 < nodes) h2 = box_hit(c1 + 1, poi, inv[l], out[l].t);
                    }
                    const int near_ok = neg ? h2 : h1, far_ok = neg ? h1 : h2;
                    if (far_ok) { slo[l][L] = nlo[l]; shi[l][L] = nhi[l]; trail[l] |= 1u << L; }
                    if (near_ok) { lo[l] = nlo[l]; hi[l] = nhi[l]; }
                    act[l] = near_ok;
                    any_near |= near_ok;
                }
                k = neg ? c1 + 1 : c1;
                lvl = L;
                ax = na;
                if (any_near) continue;
            }
        }
        uint32_t wt = 0;
        for (int l = 0; l < 32; ++l) wt |= trail[l];
        if (wt == 0) return;
        const uint32_t L = 31u - (uint32_t)__builtin_clz(wt);
        k = (((k + 1u) >> (lvl - L)) ^ 1u) - 1u;
        lvl = L;
        ax = L % 3u;
        for (int l = 0; l < 32; ++l) {
            act[l] = (trail[l] >> L) & 1u;
            if (act[l]) { trail[l] &= ~(1u << L); lo[l] = slo[l][L]; hi[l] = shi[l][L]; }
        }
    }
}

static int same(Hit a, Hit b) {
    return a.best == b.best && bits(a.t) == bits(b.t) && bits(a.u) == bits(b.u) && bits(a.v) == bits(b.v);
}

static void* slurp(const char* path, size_t bytes) {
    FILE* f = fopen(path, "rb");
    if (!f) { perror(path); exit(2); }
    void* p = malloc(bytes);
    if (fread(p, 1, bytes, f) != bytes) { fprintf(stderr, "short read %s\n", path); exit(2); }
    fclose(f);
    return p;
}

int main(int argc, char** argv) {
    if (argc != 6) return 2;
    count = (uint32_t)atoi(argv[4]);
    const uint32_t n = (uint32_t)atoi(argv[5]);
    nodes = count / 2;
    V = slurp(argv[1], (size_t)count * 36);
    perm = slurp(argv[2], (size_t)count * 4);
    const float* R = slurp(argv[3], (size_t)n * 32);
    /* subtree boxes bottom up (the pair's box and the children's), then
     * padded as the build pads the children's boxes in a node's record */
    float* sb = malloc(24 * (size_t)nodes);
    box = malloc(24 * (size_t)nodes);
    for (uint32_t k = nodes; k-- > 0;) {
        float* b = sb + 6 * (size_t)k;
        for (uint32_t a = 0; a < 3; ++a) slab(k, a, &b[a], &b[3 + a]);
        for (uint32_t j = 1; j <= 2; ++j) {
            const uint32_t c = 2 * k + j;
            if (c >= nodes) continue;
            const float* cb = sb + 6 * (size_t)c;
            for (uint32_t a = 0; a < 3; ++a) { b[a] = fminf(b[a], cb[a]); b[3 + a] = fmaxf(b[3 + a], cb[3 + a]); }
        }
        for (uint32_t a = 0; a < 3; ++a) {
            const float pd = 1e-5f * (fabsf(b[a]) + fabsf(b[3 + a])) + 1e-30f;
            box[6 * (size_t)k + a] = b[a] - pd;
            box[6 * (size_t)k + 3 + a] = b[3 + a] + pd;
        }
    }
    uint32_t bad = 0;
    for (uint32_t c0 = 0; c0 + 32 <= n; c0 += 32) {
        f3 p[32], d[32];
        float tm[32];
        for (int l = 0; l < 32; ++l) {
            const float* r = R + 8 * (size_t)(c0 + l);
            p[l].x = r[0]; p[l].y = r[1]; p[l].z = r[2]; tm[l] = r[3];
            d[l].x = r[4]; d[l].y = r[5]; d[l].z = r[6];
        }
        const uint32_t oct = (d[0].x < 0.0f ? 1u : 0u) | (d[0].y < 0.0f ? 2u : 0u) | (d[0].z < 0.0f ? 4u : 0u);
        for (int any = 0; any < 2; ++any) {
            Hit pk[32];
            packet(any, p, d, tm, oct, pk);
            for (int l = 0; l < 32; ++l) {
                const Hit ref = reference(any, p[l], d[l], tm[l]);
                const Hit pl = per_lane(any, p[l], d[l], tm[l]);
                /* any hit reports only the occluder (intersectAny returns on the first hit) */
                const int ok = any ? (pk[l].best == ref.best && pl.best == ref.best)
                                   : (same(pk[l], ref) && same(pl, ref));
                if (!ok) {
                    if (bad < 5)
                        fprintf(stderr, "ray %u any=%d ref %u pl %u pk %u\n", c0 + l, any, ref.best, pl.best, pk[l].best);
                    ++bad;
                }
            }
        }
    }
    printf("%u %u\n", n, bad);
    return bad ? 1 : 0;
}
