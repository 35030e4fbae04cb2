// bg_traverse.cuh - closest-hit and any-hit traversal of the two BVH layouts.
//
// RefBVH: the reference's binary BVH exactly as BVH::intersect / intersect_test walk it
// (src/accelerators/bvh.rs:281-423): same node order, near child first by the sign of the
// direction along the split axis, PBRT's robust slab test (src/geometries/bounds3.rs:246-288),
// leaf primitives in ordered_primitives order, a hit at t == t_max replacing the previous one.
// REF_COMPAT renders need this walk: whether the same camera ray re-hits its surface (the
// reference never re-spawns its path, src/integrators/path.rs:70-143) depends on the exact leaf
// bounds the slab test sees.
//
// Bvh2: the library's own 2-wide BVH (both child boxes stored in the parent, 64 B nodes read as
// four 128-bit loads) for PBRT-mode rendering and the ray-query entry points.  Slab test uses
// fma with a precomputed origin * inv_dir and the same (1 + 2*gamma(3)) far-bound enlargement.
#pragma once
#include "bg_device.h"
#include "bg_math.cuh"
#include "bg_shapes.cuh"

namespace bg {

// ---------------------------------------------------------------- reference layout
BG_D bool ref_slab(const RefNode& nd, const Ray& ray, V3 inv, const int neg[3]) {
    const float k = 1.0f + 2.0f * gamma(3.0f);
    float bx0 = neg[0] ? nd.mx[0] : nd.mn[0], bx1 = neg[0] ? nd.mn[0] : nd.mx[0];
    float by0 = neg[1] ? nd.mx[1] : nd.mn[1], by1 = neg[1] ? nd.mn[1] : nd.mx[1];
    float bz0 = neg[2] ? nd.mx[2] : nd.mn[2], bz1 = neg[2] ? nd.mn[2] : nd.mx[2];
    float t_min = (bx0 - ray.o.x) * inv.x;
    float t_max = (bx1 - ray.o.x) * inv.x;
    float ty_min = (by0 - ray.o.y) * inv.y;
    float ty_max = (by1 - ray.o.y) * inv.y;
    t_max *= k;
    ty_max *= k;
    if (t_min > ty_max || ty_min > t_max) return false;
    if (ty_min > t_min) t_min = ty_min;
    if (ty_max < t_max) t_max = ty_max;
    float tz_min = (bz0 - ray.o.z) * inv.z;
    float tz_max = (bz1 - ray.o.z) * inv.z;
    tz_max *= k;
    if (t_min > tz_max || tz_min > t_max) return false;
    if (tz_min > t_min) t_min = tz_min;
    if (tz_max < t_max) t_max = tz_max;
    return (t_min < ray.t_max) && (t_max > 0.0f);
}

// Primitive test against the current t_max; updates ray.t_max on a closest hit.
BG_D bool prim_hit(const Scene& sc, uint32_t prim, const TriRay& tr, Ray& ray, bool closest) {
    if (prim < sc.ntri) {
        V3 p0, p1, p2;
        load_tri(sc, prim, &p0, &p1, &p2);
        TriHit h;
        if (!tri_test(tr, ray.t_max, p0, p1, p2, &h)) return false;
        if (closest) ray.t_max = h.t;
        return true;
    }
    if (prim < sc.ntri + sc.nsph) {
        SphHit h;
        if (!sphere_test(sc.sph[prim - sc.ntri], ray, ray.t_max, closest ? &h : nullptr)) return false;
        if (closest) ray.t_max = h.t;
        return true;
    }
    float t;
    if (!quadric_hit(sc.quads + QUADRIC_F4 * (prim - sc.ntri - sc.nsph), ray, ray.t_max, &t, nullptr)) return false;
    if (closest) ray.t_max = t;
    return true;
}

// BVH::intersect: returns the hit prim (or -1) and leaves the hit distance in ray.t_max.
// counters (optional): [0] node visits, [1] primitive tests.
template <bool ANY>
BG_D int ref_traverse(const Scene& sc, Ray& ray, uint32_t* err, unsigned long long* counters) {
    if (sc.ref_nnodes == 0) return -1;
    V3 inv = v3(1.0f / ray.d.x, 1.0f / ray.d.y, 1.0f / ray.d.z);
    int neg[3] = {inv.x < 0.0f, inv.y < 0.0f, inv.z < 0.0f};
    TriRay tr = make_tri_ray(ray);
    uint32_t stack[TRAVERSAL_STACK];
    int sp = 0;
    uint32_t cur = 0;
    int hit = -1;
    unsigned long long visits = 0, tests = 0;
    for (;;) {
        if (cur >= sc.ref_nnodes) {
            atomicOr(err, ERR_BAD_NODE);
            break;
        }
        const RefNode nd = sc.ref_nodes[cur];
        ++visits;
        uint32_t count = nd.count_axis >> 2;
        if (ref_slab(nd, ray, inv, neg)) {
            if (count > 0) {
                for (uint32_t i = 0; i < count; ++i) {
                    uint32_t prim = sc.ref_order[nd.offset + i];
                    ++tests;
                    if (prim_hit(sc, prim, tr, ray, !ANY)) {
                        hit = (int)prim;
                        if (ANY) goto done;
                    }
                }
                if (sp == 0) break;
                cur = stack[--sp];
            } else {
                if (sp >= TRAVERSAL_STACK) {
                    atomicOr(err, ERR_STACK_OVERFLOW);
                    hit = -1;
                    break;
                }
                if (neg[nd.count_axis & 3]) {
                    stack[sp++] = cur + 1;
                    cur = nd.offset;
                } else {
                    stack[sp++] = nd.offset;
                    cur = cur + 1;
                }
            }
        } else {
            if (sp == 0) break;
            cur = stack[--sp];
        }
    }
done:
    if (counters) {
        atomicAdd(&counters[0], visits);
        atomicAdd(&counters[1], tests);
    }
    return hit;
}

// ---------------------------------------------------------------- 2-wide layout
struct FastRay {
    V3 inv, oi;  // 1/d and o/d (so t = fma(b, inv, -oi))
};
BG_D float safe_dir(float d) { return fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d); }
BG_D FastRay make_fast_ray(const Ray& r) {
    FastRay f;
    f.inv = v3(1.0f / safe_dir(r.d.x), 1.0f / safe_dir(r.d.y), 1.0f / safe_dir(r.d.z));
    f.oi = v3(r.o.x * f.inv.x, r.o.y * f.inv.y, r.o.z * f.inv.z);
    return f;
}
// Returns entry distance, or +inf on a miss (the box must start before t_max and end after 0).
BG_D float box_enter(float lox, float hix, float loy, float hiy, float loz, float hiz, const FastRay& f,
                     float t_max) {
    const float k = 1.0f + 2.0f * gamma(3.0f);
    float tx0 = fmaf(lox, f.inv.x, -f.oi.x), tx1 = fmaf(hix, f.inv.x, -f.oi.x);
    float ty0 = fmaf(loy, f.inv.y, -f.oi.y), ty1 = fmaf(hiy, f.inv.y, -f.oi.y);
    float tz0 = fmaf(loz, f.inv.z, -f.oi.z), tz1 = fmaf(hiz, f.inv.z, -f.oi.z);
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1)) * k;
    return (tn <= tf && tn < t_max) ? tn : INFINITY;
}

// Leaf slot: triangle = (p0, id) (p1, -) (p2, -); sphere = (center, id | SPHERE_BIT) (radius, -, -, -);
// quadric = (-, -, -, id | QUADRIC_BIT), the record itself lives in sc.quads.
BG_D bool leaf_prim_hit(const Scene& sc, uint32_t slot, const TriRay& tr, Ray& ray, bool closest, int* prim) {
    float4 a = __ldg(&sc.leaf_prims[3 * slot]);
    float4 b = __ldg(&sc.leaf_prims[3 * slot + 1]);
    uint32_t id = __float_as_uint(a.w);
    if (id & QUADRIC_BIT) {
        uint32_t qi = id & ~QUADRIC_BIT;
        float t;
        if (!quadric_hit(sc.quads + QUADRIC_F4 * qi, ray, ray.t_max, &t, nullptr)) return false;
        if (closest) ray.t_max = t;
        *prim = (int)(qi + sc.ntri + sc.nsph);
        return true;
    }
    if (!(id & SPHERE_BIT)) {
        float4 c = __ldg(&sc.leaf_prims[3 * slot + 2]);
        TriHit h;
        if (!tri_test(tr, ray.t_max, f4xyz(a), f4xyz(b), f4xyz(c), &h)) return false;
        if (closest) ray.t_max = h.t;
        *prim = (int)id;
        return true;
    }
    SphHit h;
    if (!sphere_test(make_float4(a.x, a.y, a.z, b.x), ray, ray.t_max, closest ? &h : nullptr)) return false;
    if (closest) ray.t_max = h.t;
    *prim = (int)(id & ~SPHERE_BIT) + (int)sc.ntri;
    return true;
}

// While-while traversal (Aila & Laine, HPG 2009) over the 2-wide layout.  Returns the hit prim
// (ANY: the first hit found) and leaves the closest distance in ray.t_max.  `skip` excludes one
// primitive (any-hit only).  Stack entries: inner node index, or a leaf as (count, ~first).
template <bool ANY>
BG_D int bvh2_traverse(const Scene& sc, Ray& ray, uint32_t* err, int skip = -1) {
    if (sc.n_nodes == 0) return -1;
    FastRay f = make_fast_ray(ray);
    TriRay tr = make_tri_ray(ray);
    int stack[TRAVERSAL_STACK];
    int sp = 0;
    int node = 0;  // >= 0: inner node to visit; -1: leaf pending; -2: nothing, pop
    int hit = -1;
    int leaf_first = 0, leaf_count = 0;
    for (;;) {
        while (node >= 0) {
            const Bvh2Node* n = sc.nodes + node;
            float4 a = __ldg(&n->c0xy), b = __ldg(&n->c1xy), c = __ldg(&n->c01z);
            int4 ch = __ldg(&n->child);
            float t0 = box_enter(a.x, a.y, a.z, a.w, c.x, c.y, f, ray.t_max);
            float t1 = box_enter(b.x, b.y, b.z, b.w, c.z, c.w, f, ray.t_max);
            bool h0 = t0 != INFINITY, h1 = t1 != INFINITY;
            if (!h0 && !h1) {
                node = -2;
                break;
            }
            int first = h0 ? ch.x : ch.y, cfirst = h0 ? ch.z : ch.w;
            if (h0 && h1) {
                int second = ch.y, csecond = ch.w;
                if (t1 < t0) {
                    first = ch.y;
                    cfirst = ch.w;
                    second = ch.x;
                    csecond = ch.z;
                }
                if (sp + 2 > TRAVERSAL_STACK) {
                    atomicOr(err, ERR_STACK_OVERFLOW);
                    return hit;
                }
                if (second < 0) stack[sp++] = csecond;
                stack[sp++] = second;
            }
            if (first < 0) {
                leaf_first = ~first;
                leaf_count = cfirst;
                node = -1;
            } else {
                node = first;
            }
        }
        if (node == -1) {
            for (int i = 0; i < leaf_count; ++i) {
                int prim;
                if (leaf_prim_hit(sc, (uint32_t)(leaf_first + i), tr, ray, !ANY, &prim)) {
                    if (ANY && prim == skip) continue;
                    hit = prim;
                    if (ANY) return hit;
                }
            }
        }
        if (sp == 0) return hit;
        int e = stack[--sp];
        if (e < 0) {
            leaf_first = ~e;
            leaf_count = stack[--sp];
            node = -1;
        } else {
            node = e;
        }
    }
}

// ---------------------------------------------------------------- persistent traversal with ray
// replacement.  Each warp keeps up to 32 rays in flight; after every traversal step (inner nodes
// down to one leaf) lanes whose ray finished store the result, and once at least kRefill lanes are
// idle the warp fetches that many new rays with one atomic (Aila & Laine, HPG 2009, dynamic
// fetch).  refill = 32 fetches only when the whole warp is idle.  Src supplies rays and takes
// results: Ray load(uint32_t i, int* skip), void store(uint32_t i, int prim, float t).
template <bool ANY, class Src>
BG_D void traverse_queue(const Scene& sc, uint32_t n, uint32_t* head, Src& src, uint32_t* err, int refill) {
    const uint32_t lane = threadIdx.x & 31u;
    int stack[TRAVERSAL_STACK];
    Ray ray;
    FastRay f;
    TriRay tr;
    int sp = 0, node = -2, hit = -1, skip = -1, leaf_first = 0, leaf_count = 0;
    uint32_t idx = 0;
    bool busy = false, exhausted = false;
    for (;;) {
        // refill idle lanes
        const unsigned idle = __ballot_sync(0xffffffffu, !busy && !exhausted);
        const int nidle = __popc(idle);
        if (nidle >= refill || (nidle > 0 && __ballot_sync(0xffffffffu, busy) == 0)) {
            const uint32_t leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(head, (uint32_t)nidle);
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!busy && !exhausted) {
                uint32_t my = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (my < n) {
                    idx = my;
                    ray = src.load(my, &skip);
                    f = make_fast_ray(ray);
                    tr = make_tri_ray(ray);
                    sp = 0;
                    node = sc.n_nodes ? 0 : -2;
                    hit = -1;
                    leaf_count = 0;
                    busy = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, busy) == 0) break;
        if (busy) {
            // inner nodes until a leaf is found or this subtree is missed
            while (node >= 0) {
                const Bvh2Node* nd = sc.nodes + node;
                float4 a = __ldg(&nd->c0xy), b = __ldg(&nd->c1xy), c = __ldg(&nd->c01z);
                int4 ch = __ldg(&nd->child);
                float t0 = box_enter(a.x, a.y, a.z, a.w, c.x, c.y, f, ray.t_max);
                float t1 = box_enter(b.x, b.y, b.z, b.w, c.z, c.w, f, ray.t_max);
                bool h0 = t0 != INFINITY, h1 = t1 != INFINITY;
                if (!h0 && !h1) {
                    node = -2;
                    break;
                }
                int first = h0 ? ch.x : ch.y, cfirst = h0 ? ch.z : ch.w;
                if (h0 && h1) {
                    int second = ch.y, csecond = ch.w;
                    if (t1 < t0) {
                        first = ch.y;
                        cfirst = ch.w;
                        second = ch.x;
                        csecond = ch.z;
                    }
                    if (sp + 2 > TRAVERSAL_STACK) {
                        atomicOr(err, ERR_STACK_OVERFLOW);
                        sp = 0;
                        node = -2;
                        break;
                    }
                    if (second < 0) stack[sp++] = csecond;
                    stack[sp++] = second;
                }
                if (first < 0) {
                    leaf_first = ~first;
                    leaf_count = cfirst;
                    node = -1;
                } else {
                    node = first;
                }
            }
            bool done = false;
            if (node == -1) {
                for (int i = 0; i < leaf_count; ++i) {
                    int prim;
                    if (leaf_prim_hit(sc, (uint32_t)(leaf_first + i), tr, ray, !ANY, &prim)) {
                        if (ANY && prim == skip) continue;
                        hit = prim;
                        if (ANY) {
                            done = true;
                            break;
                        }
                    }
                }
                leaf_count = 0;
            }
            if (!done) {
                if (sp == 0) {
                    done = true;
                } else {
                    int e = stack[--sp];
                    if (e < 0) {
                        leaf_first = ~e;
                        leaf_count = stack[--sp];
                        node = -1;
                    } else {
                        node = e;
                    }
                }
            }
            if (done) {
                src.store(idx, hit, ray.t_max);
                busy = false;
            }
        }
    }
}

// ---------------------------------------------------------------- 8-wide compressed layout
// Traversal of Bvh8Node trees (Ylitie, Karras, Laine, HPG 2017): a node group (child_base,
// hit bits) stays in registers; the upper 8 hit bits are internal children in octant order
// (bit 24 + (slot ^ octinv)), so the highest bit is the nearest child for this ray's direction;
// the lower 24 bits are leaf primitives relative to tri_base.  The stack holds node groups only.
constexpr int STACK8 = 32;
#ifndef BG_SMEM_STACK
#define BG_SMEM_STACK 0
#endif

BG_D uint32_t sign_extend_bytes(uint32_t x) { return ((x & 0x80808080u) >> 7) * 0xFFu; }
// Byte j of w as a float: one byte permute builds 0x4B0000bb = 2^23 + b, one exact subtraction
// (BG_BYTE_PERM=0: shift, mask and integer conversion instead).
#ifndef BG_BYTE_PERM
#define BG_BYTE_PERM 0
#endif
BG_D float byte_as_float(uint32_t w, int j) {
#if BG_BYTE_PERM
    const uint32_t sel = (uint32_t)j | (4u << 4) | (5u << 8) | (7u << 12);
    return __uint_as_float(__byte_perm(w, 0x4B000000u, sel)) - 8388608.0f;
#else
    return (float)((w >> (8 * j)) & 0xFFu);
#endif
}

struct Ray8 {
    V3 o;
    V3 idir;
    uint32_t octinv4;
    bool negx, negy, negz;
};
BG_D Ray8 make_ray8(const Ray& r) {
    Ray8 q;
    q.o = r.o;
    q.idir = v3(1.0f / safe_dir(r.d.x), 1.0f / safe_dir(r.d.y), 1.0f / safe_dir(r.d.z));
    q.negx = r.d.x < 0.0f;
    q.negy = r.d.y < 0.0f;
    q.negz = r.d.z < 0.0f;
    uint32_t oct = (q.negx ? 4u : 0u) | (q.negy ? 2u : 0u) | (q.negz ? 1u : 0u);
    q.octinv4 = (7u - oct) * 0x01010101u;
    return q;
}

// Bit j of x moves to bit j ^ o (o < 8): the ray's octant order of the eight child slots.
BG_HD uint32_t octant_permute(uint32_t x, uint32_t o) {
    if (o & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
    if (o & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
    if (o & 4u) x = ((x & 0x0Fu) << 4) | ((x >> 4) & 0x0Fu);
    return x;
}

// The octant permutations of every 8-bit mask, perm[o * 256 + x] = octant_permute(x, o), in shared
// memory for the persistent traversal (one lookup per node instead of three swap stages).
BG_D void octant_table_fill(uint8_t* perm) {
    for (uint32_t i = threadIdx.x; i < 2048u; i += blockDim.x) perm[i] = (uint8_t)octant_permute(i & 255u, i >> 8);
}

// Intersects the 8 child boxes of node `ni`.  Node group: (child_base, hit internal children in
// bits 24-31 in this ray's octant order | imask); primitive group: (tri_base, hit leaves (bits 0-7,
// slot order) | leafmask << 8 | twomask << 16).  perm: the shared octant table, or null.
BG_D void bvh8_node_hits(const Scene& sc, uint32_t ni, const Ray8& r, float t_max, const uint8_t* perm,
                         uint2* ngroup, uint2* tgroup) {
    const float4* raw = reinterpret_cast<const float4*>(sc.nodes8 + ni);
    const float4 n0 = __ldg(raw + 0), n1 = __ldg(raw + 1), n2 = __ldg(raw + 2), n3 = __ldg(raw + 3),
                 n4 = __ldg(raw + 4);
    const uint32_t ebits = __float_as_uint(n0.w);
    const float sx = __uint_as_float((ebits & 0xFFu) << 23);
    const float sy = __uint_as_float(((ebits >> 8) & 0xFFu) << 23);
    const float sz = __uint_as_float(((ebits >> 16) & 0xFFu) << 23);
    const uint32_t imask = ebits >> 24;
    const V3 aidir = v3(sx * r.idir.x, sy * r.idir.y, sz * r.idir.z);
    const V3 aorig = v3((n0.x - r.o.x) * r.idir.x, (n0.y - r.o.y) * r.idir.y, (n0.z - r.o.z) * r.idir.z);
    const uint32_t qlx[2] = {__float_as_uint(n2.x), __float_as_uint(n2.y)};
    const uint32_t qly[2] = {__float_as_uint(n2.z), __float_as_uint(n2.w)};
    const uint32_t qlz[2] = {__float_as_uint(n3.x), __float_as_uint(n3.y)};
    const uint32_t qhx[2] = {__float_as_uint(n3.z), __float_as_uint(n3.w)};
    const uint32_t qhy[2] = {__float_as_uint(n4.x), __float_as_uint(n4.y)};
    const uint32_t qhz[2] = {__float_as_uint(n4.z), __float_as_uint(n4.w)};
    const float k = 1.0f + 2.0f * gamma(3.0f);
    uint32_t h = 0;  // bit s: the box of slot s is entered within [0, t_max]
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        // near / far planes per axis by the sign of the direction
        const uint32_t nx = r.negx ? qhx[i] : qlx[i], fx = r.negx ? qlx[i] : qhx[i];
        const uint32_t ny = r.negy ? qhy[i] : qly[i], fy = r.negy ? qly[i] : qhy[i];
        const uint32_t nz = r.negz ? qhz[i] : qlz[i], fz = r.negz ? qlz[i] : qhz[i];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float tnx = fmaf(byte_as_float(nx, j), aidir.x, aorig.x);
            const float tny = fmaf(byte_as_float(ny, j), aidir.y, aorig.y);
            const float tnz = fmaf(byte_as_float(nz, j), aidir.z, aorig.z);
            const float tfx = fmaf(byte_as_float(fx, j), aidir.x, aorig.x);
            const float tfy = fmaf(byte_as_float(fy, j), aidir.y, aorig.y);
            const float tfz = fmaf(byte_as_float(fz, j), aidir.z, aorig.z);
            const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.0f));
            const float tf = fminf(fminf(fminf(tfx, tfy), tfz) * k, t_max);
            if (tn <= tf) h |= 1u << (4 * i + j);
        }
    }
    const uint32_t inner = h & imask;
    const uint32_t oct = r.octinv4 & 7u;
    const uint32_t ordered = perm ? (uint32_t)perm[oct * 256u + inner] : octant_permute(inner, oct);
    const uint32_t lw = __float_as_uint(n1.z) & 0xFFFFu;  // leafmask | twomask << 8
    ngroup->x = __float_as_uint(n1.x);  // child_base
    ngroup->y = (ordered << 24) | imask;
    tgroup->x = __float_as_uint(n1.y);  // tri_base
    tgroup->y = (h & lw & 0xFFu) | (lw << 8);
}

// Next primitive of a primitive group (its hit-leaf bits must not be empty): the highest hit slot
// first; of a leaf with two primitives the second first (its twomask bit then clears, which leaves
// the offsets of the lower slots unchanged).  Returns the primitive's index in leaf_prims.
BG_D uint32_t next_leaf_prim(uint2& tg) {
    const uint32_t j = 31u - __clz(tg.y & 0xFFu);
    const uint32_t below = (1u << j) - 1u;
    uint32_t pi = tg.x + __popc((tg.y >> 8) & below) + __popc((tg.y >> 16) & below);
    if ((tg.y >> (16 + j)) & 1u) {
        pi += 1u;
        tg.y &= ~(1u << (16 + j));
    } else {
        tg.y &= ~(1u << j);
    }
    return pi;
}

// One ray through the 8-wide layout on one thread (the node-group walk of traverse_queue8 without
// the warp's ray replacement), for the per-sample megakernels.  Returns the hit prim; closest hit
// leaves the distance in ray.t_max.  `skip` excludes one primitive (any-hit only).
template <bool ANY>
BG_D int bvh8_traverse(const Scene& sc, Ray& ray, uint32_t* err, int skip = -1) {
    if (sc.n_nodes8 == 0) return -1;
    const Ray8 r8 = make_ray8(ray);
    const TriRay tr = make_tri_ray(ray);
    uint2 stack[STACK8];
    int sp = 0, hit = -1;
    uint2 ngroup = make_uint2(0, 0x80000000u), tgroup = make_uint2(0, 0);
    for (;;) {
        if (ngroup.y > 0x00FFFFFFu) {
            const uint32_t hits = ngroup.y;
            const uint32_t bit = 31u - __clz(hits);
            ngroup.y &= ~(1u << bit);
            if (ngroup.y > 0x00FFFFFFu) {
                if (sp >= STACK8) {
                    atomicOr(err, ERR_STACK_OVERFLOW);
                    return hit;
                }
                stack[sp++] = ngroup;
            }
            const uint32_t slot = (bit - 24u) ^ (r8.octinv4 & 0xFFu);
            const uint32_t rel = __popc(hits & ~(0xFFFFFFFFu << slot));
            const uint32_t child = ngroup.x + rel;
            if (child >= sc.n_nodes8) {
                atomicOr(err, ERR_BAD_NODE);
                return hit;
            }
            bvh8_node_hits(sc, child, r8, ray.t_max, nullptr, &ngroup, &tgroup);
        }
        while (tgroup.y & 0xFFu) {
            const uint32_t pi = next_leaf_prim(tgroup);
            if (pi >= sc.ntri + sc.nsph + sc.nquad) {
                atomicOr(err, ERR_BAD_PRIM);
                continue;
            }
            int prim;
            if (leaf_prim_hit(sc, pi, tr, ray, !ANY, &prim)) {
                if (ANY && prim == skip) continue;
                hit = prim;
                if (ANY) return hit;
            }
        }
        if (ngroup.y <= 0x00FFFFFFu) {
            if (sp == 0) return hit;
            ngroup = stack[--sp];
        }
    }
}

// Persistent traversal of the 8-wide layout with in-warp ray replacement (see traverse_queue).
// Each iteration a lane visits at most one node (the next child of its node group) and tests at
// most one primitive of its pending primitive group.  A node test that yields primitives while
// others are still pending pushes them (a primitive group: upper byte 0) behind the pending ones.
// Testing a whole group in one iteration would hold the warp for as many steps as its largest group
// while the other lanes wait; interleaving keeps the primitive steps as full as the node steps.
// The node-group stack lives in local memory (BG_SMEM_STACK: shared memory, entry k of thread t at
// smem[k * blockDim.x + t]).
// MULTI: rays of different scenes share the queue; src.scene(i) gives the scene of ray i.
template <bool ANY, class Src, bool MULTI = false>
BG_D void traverse_queue8(const Scene& sc, uint32_t n, uint32_t* head, Src& src, uint32_t* err, int refill,
                          uint2* smem) {
    const Scene* cur = nullptr;  // MULTI: scene of this lane's ray
    auto S = [&]() -> const Scene& {
        if constexpr (MULTI) return *cur;
        else return sc;
    };
    const uint32_t lane = threadIdx.x & 31u;
    __shared__ uint8_t octant_perm[2048];
    octant_table_fill(octant_perm);
    __syncthreads();
#if BG_SMEM_STACK
    uint2* stack = smem + threadIdx.x;
    const uint32_t sstride = blockDim.x;
#else
    uint2 stack[STACK8];
    const uint32_t sstride = 1;
    (void)smem;
#endif
    Ray ray;
    Ray8 r8;
    TriRay tr;
    uint2 ngroup = make_uint2(0, 0), tgroup = make_uint2(0, 0);
    int sp = 0, hit = -1, skip = -1;
    uint32_t idx = 0;
    bool busy = false, exhausted = false;
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !busy && !exhausted);
        const int nidle = __popc(idle);
        if (nidle >= refill || (nidle > 0 && __ballot_sync(0xffffffffu, busy) == 0)) {
            const uint32_t leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(head, (uint32_t)nidle);
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!busy && !exhausted) {
                uint32_t my = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (my < n) {
                    idx = my;
                    ray = src.load(my, &skip);
                    if constexpr (MULTI) cur = src.scene(my);
                    r8 = make_ray8(ray);
                    tr = make_tri_ray(ray);
                    sp = 0;
                    hit = -1;
                    ngroup = make_uint2(0, S().n_nodes8 ? 0x80000000u : 0u);
                    tgroup = make_uint2(0, 0);
                    busy = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, busy) == 0) break;
        if (!busy) continue;
        bool done = false;
        // node step: the next child of the node group (room for two pushes when primitives wait)
        if (ngroup.y > 0x00FFFFFFu && ((tgroup.y & 0xFFu) == 0 || sp + 2 <= STACK8)) {
            const uint32_t hits = ngroup.y;
            const uint32_t bit = 31u - __clz(hits);
            ngroup.y &= ~(1u << bit);
            if (ngroup.y > 0x00FFFFFFu) {
                if (sp >= STACK8) {
                    atomicOr(err, ERR_STACK_OVERFLOW);
                    sp = 0;
                    ngroup.y = 0;
                } else {
                    stack[sstride * sp++] = ngroup;
                }
            }
            const uint32_t slot = (bit - 24u) ^ (r8.octinv4 & 0xFFu);
            const uint32_t rel = __popc(hits & ~(0xFFFFFFFFu << slot));
            const uint32_t child = ngroup.x + rel;
            if (child >= S().n_nodes8) {
                atomicOr(err, ERR_BAD_NODE);
                sp = 0;
                ngroup = make_uint2(0, 0);
                tgroup = make_uint2(0, 0);
            } else {
                uint2 found;
                bvh8_node_hits(S(), child, r8, ray.t_max, octant_perm, &ngroup, &found);
                if (found.y & 0xFFu) {
                    if ((tgroup.y & 0xFFu) == 0) tgroup = found;
                    else stack[sstride * sp++] = found;  // upper byte 0: a primitive group
                }
            }
        }
        // primitive step: one primitive of the pending group
        if (tgroup.y & 0xFFu) {
            const uint32_t pi = next_leaf_prim(tgroup);
            if (pi >= S().ntri + S().nsph + S().nquad) {
                atomicOr(err, ERR_BAD_PRIM);
            } else {
                int prim;
                if (leaf_prim_hit(S(), pi, tr, ray, !ANY, &prim) && !(ANY && prim == skip)) {
                    hit = prim;
                    if (ANY) done = true;
                }
            }
        }
        // next groups: a node group from the stack; a primitive group only when none is pending
        if (!done && ngroup.y <= 0x00FFFFFFu) {
            while (sp > 0) {
                const uint2 g = stack[sstride * (sp - 1)];
                if (g.y > 0x00FFFFFFu) {
                    ngroup = g;
                    --sp;
                        break;
                }
                if (tgroup.y & 0xFFu) break;
                tgroup = g;
                --sp;
            }
            if (ngroup.y <= 0x00FFFFFFu && (tgroup.y & 0xFFu) == 0 && sp == 0) done = true;
        }
        if (done) {
            src.store(idx, hit, ray.t_max);
            busy = false;
        }
    }
}

}  // namespace bg
