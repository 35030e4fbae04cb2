// bg_bvh.cpp - host BVH builders (reference layout and the 2-wide layout).
// Built with -ffp-contract=off so the reference build's f32 SAH arithmetic rounds as in Rust.
#include "bg_bvh.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <deque>
#include <future>
#include <memory>

namespace bg {

namespace {

struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const Box& b) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::fmin(lo[i], b.lo[i]);
            hi[i] = std::fmax(hi[i], b.hi[i]);
        }
    }
    void grow(const float* p) {
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::fmin(lo[i], p[i]);
            hi[i] = std::fmax(hi[i], p[i]);
        }
    }
    float area() const {  // Bounds3::surface_area (bounds3.rs:160-163)
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dx * dz + dy * dz);
    }
    int max_extent() const {  // Bounds3::maximum_extent (bounds3.rs:175-184)
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx > dy && dx > dz) return 0;
        if (dy > dz) return 1;
        return 2;
    }
};

// Primitive bounds as the reference computes them: Triangle::world_bounds (triangle.rs:128-133);
// Sphere::world_bounds = object_to_world.transform_bounds(object bounds) (sphere.rs:68-78,
// transform.rs:75-86) with object_to_world = translate(center).
Box prim_box(const HostPrims& p, uint32_t i) {
    Box b;
    if (i < p.ntri) {
        const float* v = p.tri + 9 * (size_t)i;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = std::fmin(v[k], v[3 + k]);
            b.hi[k] = std::fmax(v[k], v[3 + k]);
        }
        b.grow(v + 6);
        return b;
    }
    float m[3][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}};
    float lo[3], hi[3];
    if (i < p.ntri + p.nsph) {
        const bg_sphere& s = p.sph[i - p.ntri];
        const float r = s.radius;
        lo[0] = -r; lo[1] = -r; lo[2] = std::fmin(-r, r);
        hi[0] = r; hi[1] = r; hi[2] = std::fmax(-r, r);
        m[0][3] = s.center[0];
        m[1][3] = s.center[1];
        m[2][3] = s.center[2];
    } else {  // cylinder.rs:61-66, disk.rs:57-62, cone.rs:57-62
        const bg_quadric& q = p.quad[i - p.ntri - p.nsph];
        const float r = q.radius;
        float z0 = 0.0f, z1 = 0.0f;
        if (q.kind == BG_QUADRIC_CYLINDER) {
            z0 = std::fmin(q.z_min, q.z_max);
            z1 = std::fmax(q.z_min, q.z_max);
        } else if (q.kind == BG_QUADRIC_DISK) {
            z0 = z1 = q.height;
        } else {
            z0 = 0.0f;
            z1 = q.height;
        }
        lo[0] = -r; lo[1] = -r; lo[2] = z0;
        hi[0] = r; hi[1] = r; hi[2] = z1;
        for (int rr = 0; rr < 3; ++rr)
            for (int c = 0; c < 4; ++c) m[rr][c] = q.object_to_world[4 * rr + c];
    }
    bool first = true;
    for (int c = 0; c < 8; ++c) {
        // corner order of transform_bounds; Point3::transform: m00*x + m01*y + m02*z + m03
        static const int order[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                        {0, 1, 1}, {1, 1, 0}, {1, 0, 1}, {1, 1, 1}};
        float q[3] = {order[c][0] ? hi[0] : lo[0], order[c][1] ? hi[1] : lo[1], order[c][2] ? hi[2] : lo[2]};
        float w[3];
        for (int k = 0; k < 3; ++k) w[k] = m[k][0] * q[0] + m[k][1] * q[1] + m[k][2] * q[2] + m[k][3];
        if (first) {
            for (int k = 0; k < 3; ++k) b.lo[k] = b.hi[k] = w[k];
            first = false;
        } else {
            b.grow(w);
        }
    }
    return b;
}

struct RefInfo {
    uint32_t index;
    Box box;
    float c[3];
};

// itertools::partition (two-pointer; elements mapping to true are moved to the front).
template <class F>
size_t two_pointer_partition(RefInfo* v, size_t n, F pred) {
    size_t front = 0, back = n, split = 0;
    while (front < back) {
        RefInfo* f = &v[front++];
        if (!pred(*f)) {
            bool swapped = false;
            while (front < back) {
                RefInfo* b = &v[--back];
                if (pred(*b)) {
                    std::swap(*f, *b);
                    swapped = true;
                    break;
                }
            }
            if (!swapped) return split;
        }
        ++split;
    }
    return split;
}

}  // namespace

void prim_bounds(const HostPrims& p, uint32_t i, float lo[3], float hi[3]) {
    Box b = prim_box(p, i);
    for (int k = 0; k < 3; ++k) {
        lo[k] = b.lo[k];
        hi[k] = b.hi[k];
    }
}

bool build_reference_bvh(const HostPrims& p, bool faithful, RefBvh* out, uint64_t max_prims_faithful) {
    const uint64_t n = p.count();
    out->nodes.clear();
    out->order.clear();
    if (n == 0) return true;
    if (faithful && n > max_prims_faithful) return false;  // O(n^2) chain build (bvh.rs:154-155)
    std::vector<RefInfo> info(n);
    for (uint32_t i = 0; i < n; ++i) {
        info[i].index = i;
        info[i].box = prim_box(p, i);
        for (int k = 0; k < 3; ++k) info[i].c[k] = 0.5f * info[i].box.lo[k] + 0.5f * info[i].box.hi[k];
    }
    out->nodes.reserve(2 * n);
    out->order.reserve(n);
    struct Task {
        size_t begin, end;
        int64_t parent;
    };
    std::vector<Task> stack{{0, (size_t)n, -1}};
    const int NB = 16;
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        uint32_t idx = (uint32_t)out->nodes.size();
        out->nodes.push_back(RefNode{});
        if (t.parent >= 0) out->nodes[t.parent].offset = idx;  // second_child_offset
        RefInfo* v = info.data() + t.begin;
        const size_t size = t.end - t.begin;
        Box bounds;
        for (size_t i = 0; i < size; ++i) bounds.grow(v[i].box);
        auto leaf = [&]() {
            RefNode& nd = out->nodes[idx];
            std::memcpy(nd.mn, bounds.lo, sizeof(nd.mn));
            std::memcpy(nd.mx, bounds.hi, sizeof(nd.mx));
            nd.offset = (uint32_t)out->order.size();
            nd.count_axis = (uint32_t)size << 2;
            for (size_t i = 0; i < size; ++i) out->order.push_back(v[i].index);
        };
        if (size == 1) {
            leaf();
            continue;
        }
        Box cb;
        for (size_t i = 0; i < size; ++i) cb.grow(v[i].c);
        const int dim = cb.max_extent();
        if (cb.hi[dim] == cb.lo[dim]) {
            leaf();
            continue;
        }
        size_t mid = size / 2;
        if (size <= 2) {
            if (v[0].c[dim] > v[1].c[dim]) std::swap(v[0], v[1]);  // select_nth_unstable_by
        } else {
            auto bucket = [&](const RefInfo& r) -> int {
                float off = r.c[dim] - cb.lo[dim];  // Bounds3::offset (bounds3.rs:194-206)
                if (cb.hi[dim] > cb.lo[dim]) off /= cb.hi[dim] - cb.lo[dim];
                size_t b;
                if (faithful) {
                    b = (size_t)NB * (off >= 1.0f ? 1u : 0u);
                } else {
                    float fb = (float)NB * off;
                    b = fb <= 0.0f ? 0 : (size_t)fb;
                }
                if (b >= (size_t)NB) b = NB - 1;
                return (int)b;
            };
            float cnt[NB] = {0};
            Box bb[NB];
            for (size_t i = 0; i < size; ++i) {
                int b = bucket(v[i]);
                cnt[b] += 1.0f;
                bb[b].grow(v[i].box);
            }
            float cost[NB - 1];
            const float sa = bounds.area();
            for (int i = 0; i < NB - 1; ++i) {
                Box b0, b1;
                float c0 = 0.0f, c1 = 0.0f;
                for (int j = 0; j <= i; ++j) {
                    b0.grow(bb[j]);
                    c0 += cnt[j];
                }
                for (int j = i + 1; j < NB; ++j) {
                    b1.grow(bb[j]);
                    c1 += cnt[j];
                }
                cost[i] = 1.0f + (c0 * b0.area() + c1 * b1.area()) / sa;
            }
            float min_cost = cost[0];
            int min_b = 0;
            for (int i = 1; i < NB - 1; ++i)
                if (cost[i] < min_cost) {
                    min_cost = cost[i];
                    min_b = i;
                }
            if (size > 256 || min_cost < (float)size) {
                mid = two_pointer_partition(v, size, [&](const RefInfo& r) { return bucket(r) <= min_b; });
            } else {
                leaf();
                continue;
            }
        }
        RefNode& nd = out->nodes[idx];
        std::memcpy(nd.mn, bounds.lo, sizeof(nd.mn));
        std::memcpy(nd.mx, bounds.hi, sizeof(nd.mx));
        nd.count_axis = (uint32_t)dim;  // count 0
        stack.push_back({t.begin + mid, t.end, (int64_t)idx});
        stack.push_back({t.begin, t.begin + mid, -1});
    }
    return true;
}

// ================================================================ 2-wide BVH
namespace {

struct Ref2 {
    float lo[3], hi[3], c[3];
    uint32_t id;
};
struct BNode {
    Box box;
    std::unique_ptr<BNode> l, r;
    uint32_t first = 0, count = 0;
};
constexpr int NBINS = 32;
constexpr float C_TRAV = 1.2f;

std::unique_ptr<BNode> build_rec(Ref2* refs, uint32_t begin, uint32_t end, int depth, uint32_t MAX_LEAF) {
    auto node = std::make_unique<BNode>();
    Box cb;
    for (uint32_t i = begin; i < end; ++i) {
        for (int k = 0; k < 3; ++k) {
            node->box.lo[k] = std::fmin(node->box.lo[k], refs[i].lo[k]);
            node->box.hi[k] = std::fmax(node->box.hi[k], refs[i].hi[k]);
        }
        cb.grow(refs[i].c);
    }
    const uint32_t n = end - begin;
    if (n == 1) {
        node->first = begin;
        node->count = 1;
        return node;
    }
    int best_axis = -1, best_bin = -1;
    float best_cost = FLT_MAX;
    const float area = node->box.area();
    for (int a = 0; a < 3; ++a) {
        float ext = cb.hi[a] - cb.lo[a];
        if (!(ext > 0.0f)) continue;
        float scale = (float)NBINS * (1.0f - 1e-6f) / ext;
        uint32_t cnt[NBINS] = {0};
        Box bb[NBINS];
        for (uint32_t i = begin; i < end; ++i) {
            int b = std::min(NBINS - 1, (int)((refs[i].c[a] - cb.lo[a]) * scale));
            cnt[b]++;
            for (int k = 0; k < 3; ++k) {
                bb[b].lo[k] = std::fmin(bb[b].lo[k], refs[i].lo[k]);
                bb[b].hi[k] = std::fmax(bb[b].hi[k], refs[i].hi[k]);
            }
        }
        float right_area[NBINS];
        uint32_t right_cnt[NBINS];
        Box acc;
        uint32_t c = 0;
        for (int b = NBINS - 1; b > 0; --b) {
            acc.grow(bb[b]);
            c += cnt[b];
            right_area[b] = c ? acc.area() : 0.0f;
            right_cnt[b] = c;
        }
        Box lacc;
        uint32_t lc = 0;
        for (int b = 0; b < NBINS - 1; ++b) {
            lacc.grow(bb[b]);
            lc += cnt[b];
            if (lc == 0 || right_cnt[b + 1] == 0) continue;
            float cost = C_TRAV + ((float)lc * lacc.area() + (float)right_cnt[b + 1] * right_area[b + 1]) / area;
            if (cost < best_cost) {
                best_cost = cost;
                best_axis = a;
                best_bin = b;
            }
        }
    }
    uint32_t mid;
    if (best_axis < 0) {
        // all centroids coincide
        if (n <= MAX_LEAF) {
            node->first = begin;
            node->count = n;
            return node;
        }
        mid = begin + n / 2;
    } else {
        if (n <= MAX_LEAF && (float)n <= best_cost) {
            node->first = begin;
            node->count = n;
            return node;
        }
        const int a = best_axis;
        const float scale = (float)NBINS * (1.0f - 1e-6f) / (cb.hi[a] - cb.lo[a]);
        Ref2* m = std::partition(refs + begin, refs + end, [&](const Ref2& r) {
            return std::min(NBINS - 1, (int)((r.c[a] - cb.lo[a]) * scale)) <= best_bin;
        });
        mid = (uint32_t)(m - refs);
        if (mid == begin || mid == end) mid = begin + n / 2;
    }
    if (n > 65536 && depth < 5) {
        auto fut = std::async(std::launch::async, build_rec, refs, mid, end, depth + 1, MAX_LEAF);
        node->l = build_rec(refs, begin, mid, depth + 1, MAX_LEAF);
        node->r = fut.get();
    } else {
        node->l = build_rec(refs, begin, mid, depth + 1, MAX_LEAF);
        node->r = build_rec(refs, mid, end, depth + 1, MAX_LEAF);
    }
    return node;
}

void emit_prim(const HostPrims& p, uint32_t id, std::vector<float4>* out) {
    float4 a, b, c;
    if (id < p.ntri) {
        const float* v = p.tri + 9 * (size_t)id;
        a.x = v[0]; a.y = v[1]; a.z = v[2];
        std::memcpy(&a.w, &id, 4);
        b.x = v[3]; b.y = v[4]; b.z = v[5]; b.w = 0.0f;
        c.x = v[6]; c.y = v[7]; c.z = v[8]; c.w = 0.0f;
    } else if (id < p.ntri + p.nsph) {
        const bg_sphere& s = p.sph[id - p.ntri];
        a.x = s.center[0]; a.y = s.center[1]; a.z = s.center[2];
        uint32_t idbits = (id - p.ntri) | SPHERE_BIT;
        std::memcpy(&a.w, &idbits, 4);
        b.x = s.radius; b.y = 0.0f; b.z = 0.0f; b.w = 0.0f;
        c.x = c.y = c.z = c.w = 0.0f;
    } else {
        a.x = a.y = a.z = 0.0f;
        uint32_t idbits = (id - p.ntri - p.nsph) | QUADRIC_BIT;
        std::memcpy(&a.w, &idbits, 4);
        b.x = b.y = b.z = b.w = 0.0f;
        c.x = c.y = c.z = c.w = 0.0f;
    }
    out->push_back(a);
    out->push_back(b);
    out->push_back(c);
}

struct Flattener {
    const HostPrims& p;
    const Ref2* refs;
    Bvh2* out;
    // Emits the leaf's primitives; returns the encoded child reference (~first) and count.
    void emit_leaf(const BNode* n, int* child, int* count) {
        uint32_t first = (uint32_t)(out->leaf_prims.size() / 3);
        for (uint32_t i = 0; i < n->count; ++i) emit_prim(p, refs[n->first + i].id, &out->leaf_prims);
        *child = ~(int)first;
        *count = (int)n->count;
    }
    int emit(const BNode* n) {  // n is an inner node
        int idx = (int)out->nodes.size();
        out->nodes.push_back(Bvh2Node{});
        const BNode* ch[2] = {n->l.get(), n->r.get()};
        int cidx[2], ccnt[2];
        for (int k = 0; k < 2; ++k) {
            if (ch[k]->count > 0) emit_leaf(ch[k], &cidx[k], &ccnt[k]);
            else {
                cidx[k] = emit(ch[k]);
                ccnt[k] = 0;
            }
        }
        Bvh2Node& nd = out->nodes[idx];
        const Box& b0 = ch[0]->box;
        const Box& b1 = ch[1]->box;
        nd.c0xy = make_float4(b0.lo[0], b0.hi[0], b0.lo[1], b0.hi[1]);
        nd.c1xy = make_float4(b1.lo[0], b1.hi[0], b1.lo[1], b1.hi[1]);
        nd.c01z = make_float4(b0.lo[2], b0.hi[2], b1.lo[2], b1.hi[2]);
        nd.child = make_int4(cidx[0], cidx[1], ccnt[0], ccnt[1]);
        return idx;
    }
};

}  // namespace

void build_bvh2(const HostPrims& p, Bvh2* out, int /*threads*/) {
    out->nodes.clear();
    out->leaf_prims.clear();
    const uint32_t n = p.count();
    if (n == 0) return;
    std::vector<Ref2> refs(n);
    for (uint32_t i = 0; i < n; ++i) {
        Box b = prim_box(p, i);
        for (int k = 0; k < 3; ++k) {
            refs[i].lo[k] = b.lo[k];
            refs[i].hi[k] = b.hi[k];
            refs[i].c[k] = 0.5f * (b.lo[k] + b.hi[k]);
        }
        refs[i].id = i;
    }
    std::unique_ptr<BNode> root = build_rec(refs.data(), 0, n, 0, 8);
    out->nodes.reserve(2 * n / 3 + 2);
    out->leaf_prims.reserve(3 * (size_t)n);
    Flattener fl{p, refs.data(), out};
    if (root->count > 0) {
        // a single leaf: root with the leaf and an empty sibling
        out->nodes.push_back(Bvh2Node{});
        int c0, n0;
        fl.emit_leaf(root.get(), &c0, &n0);
        Bvh2Node& nd = out->nodes[0];
        const Box& b = root->box;
        nd.c0xy = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
        nd.c1xy = nd.c0xy;
        nd.c01z = make_float4(b.lo[2], b.hi[2], b.lo[2], b.hi[2]);
        nd.child = make_int4(c0, c0, n0, 0);
    } else {
        fl.emit(root.get());
    }
}

}  // namespace bg

// ================================================================ 8-wide compressed BVH
namespace bg {

namespace {

struct Wide {
    const BNode* bin;  // binary node whose subtree this wide node covers
    uint32_t index;
};

// Quantisation exponent of one axis: the smallest e with extent / 2^e <= 255.
int axis_exponent(double extent) {
    if (!(extent > 0.0)) return -100;
    int e = (int)std::ceil(std::log2(extent / 255.0));
    while (extent / std::ldexp(1.0, e) > 255.0) ++e;
    if (e < -100) e = -100;
    if (e > 100) e = 100;
    return e;
}

}  // namespace

bool g_bvh8_single_leaves = false;
uint32_t g_bvh8_max_leaf = 3;  // experiment: every leaf child holds one primitive
void build_bvh8(const HostPrims& p, Bvh8* out) {
    out->nodes.clear();
    out->leaf_prims.clear();
    const uint32_t n = p.count();
    if (n == 0) return;
    std::vector<Ref2> refs(n);
    for (uint32_t i = 0; i < n; ++i) {
        Box b = prim_box(p, i);
        for (int k = 0; k < 3; ++k) {
            refs[i].lo[k] = b.lo[k];
            refs[i].hi[k] = b.hi[k];
            refs[i].c[k] = 0.5f * (b.lo[k] + b.hi[k]);
        }
        refs[i].id = i;
    }
    std::unique_ptr<BNode> root = build_rec(refs.data(), 0, n, 0, 2);
    out->nodes.reserve(n / 4 + 2);
    out->leaf_prims.reserve(3 * (size_t)n);
    out->nodes.push_back(Bvh8Node{});
    std::vector<Wide> queue{{root.get(), 0}};
    std::deque<BNode> pieces;  // leaves split to fill free child slots (stable addresses)
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const BNode* b = queue[qi].bin;
        const uint32_t idx = queue[qi].index;
        // children: open the largest-area internal child until there are 8
        std::vector<const BNode*> ch;
        if (b->count > 0) ch.push_back(b);
        else {
            ch.push_back(b->l.get());
            ch.push_back(b->r.get());
            while (ch.size() < 8) {
                int best = -1;
                float best_area = -1.0f;
                for (size_t i = 0; i < ch.size(); ++i)
                    if (ch[i]->count == 0 && ch[i]->box.area() > best_area) {
                        best_area = ch[i]->box.area();
                        best = (int)i;
                    }
                if (best < 0) break;
                const BNode* c = ch[best];
                ch[best] = c->l.get();
                ch.push_back(c->r.get());
            }
        }
        // free slots: split leaves of several primitives (largest area first) so that each part
        // gets its own quantised box, which the node test culls before any primitive test
        while (ch.size() < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (size_t i = 0; i < ch.size(); ++i)
                if (ch[i]->count > 1 && ch[i]->box.area() > best_area) {
                    best_area = ch[i]->box.area();
                    best = (int)i;
                }
            if (best < 0) break;
            const BNode* c = ch[best];
            // two leaves of one primitive each
            BNode& a = pieces.emplace_back();
            BNode& r = pieces.emplace_back();
            a.first = c->first;
            a.count = 1;
            r.first = c->first + 1;
            r.count = c->count - 1;
            for (int k = 0; k < 3; ++k) {
                a.box.lo[k] = refs[a.first].lo[k];
                a.box.hi[k] = refs[a.first].hi[k];
            }
            for (uint32_t t = r.first; t < r.first + r.count; ++t)
                for (int k = 0; k < 3; ++k) {
                    r.box.lo[k] = std::fmin(r.box.lo[k], refs[t].lo[k]);
                    r.box.hi[k] = std::fmax(r.box.hi[k], refs[t].hi[k]);
                }
            ch[best] = &a;
            ch.push_back(&r);
        }
        Box nb;
        for (const BNode* c : ch) nb.grow(c->box);
        // octant slot assignment: slot s takes a child that comes first along direction d_s
        // (components negative where bits 2,1,0 of s are set), greedy on cost = <c - c_parent, d_s>
        double pc[3];
        for (int k = 0; k < 3; ++k) pc[k] = 0.5 * ((double)nb.lo[k] + nb.hi[k]);
        double cost[8][8];
        for (size_t i = 0; i < ch.size(); ++i) {
            double cc[3];
            for (int k = 0; k < 3; ++k) cc[k] = 0.5 * ((double)ch[i]->box.lo[k] + ch[i]->box.hi[k]) - pc[k];
            for (int sl = 0; sl < 8; ++sl) {
                double d[3] = {(sl & 4) ? -1.0 : 1.0, (sl & 2) ? -1.0 : 1.0, (sl & 1) ? -1.0 : 1.0};
                cost[i][sl] = cc[0] * d[0] + cc[1] * d[1] + cc[2] * d[2];
            }
        }
        int slot_child[8];
        for (int& v : slot_child) v = -1;
        std::vector<bool> assigned(ch.size(), false);
        for (size_t round = 0; round < ch.size(); ++round) {
            double best = 1e300;
            int bi = -1, bs = -1;
            for (size_t i = 0; i < ch.size(); ++i) {
                if (assigned[i]) continue;
                for (int sl = 0; sl < 8; ++sl)
                    if (slot_child[sl] < 0 && cost[i][sl] < best) {
                        best = cost[i][sl];
                        bi = (int)i;
                        bs = sl;
                    }
            }
            assigned[bi] = true;
            slot_child[bs] = bi;
        }
        Bvh8Node nd{};
        int ex[3];
        for (int k = 0; k < 3; ++k) {
            nd.p[k] = nb.lo[k];
            ex[k] = axis_exponent((double)nb.hi[k] - (double)nb.lo[k]);
            nd.e[k] = (uint8_t)(ex[k] + 127);
        }
        // internal children contiguous from child_base, leaf primitives from tri_base, both in slot
        // order; empty slots keep the inverted box (qlo 255 > qhi 0), which no ray enters
        nd.child_base = (uint32_t)(queue.size());
        nd.tri_base = (uint32_t)(out->leaf_prims.size() / 3);
        uint32_t int_k = 0;
        for (int sl = 0; sl < 8; ++sl) {
            int ci = slot_child[sl];
            if (ci < 0) {
                nd.qlo_x[sl] = nd.qlo_y[sl] = nd.qlo_z[sl] = 255;
                nd.qhi_x[sl] = nd.qhi_y[sl] = nd.qhi_z[sl] = 0;
                continue;
            }
            const BNode* c = ch[ci];
            for (int k = 0; k < 3; ++k) {
                double sc = std::ldexp(1.0, ex[k]);
                double lo = std::floor(((double)c->box.lo[k] - (double)nd.p[k]) / sc);
                double hi = std::ceil(((double)c->box.hi[k] - (double)nd.p[k]) / sc);
                uint8_t qlo = (uint8_t)std::min(255.0, std::max(0.0, lo));
                uint8_t qhi = (uint8_t)std::min(255.0, std::max(0.0, hi));
                uint8_t* dlo = k == 0 ? nd.qlo_x : (k == 1 ? nd.qlo_y : nd.qlo_z);
                uint8_t* dhi = k == 0 ? nd.qhi_x : (k == 1 ? nd.qhi_y : nd.qhi_z);
                dlo[sl] = qlo;
                dhi[sl] = qhi;
            }
            if (c->count == 0) {
                nd.imask |= (uint8_t)(1u << sl);
                queue.push_back({c, nd.child_base + int_k});
                ++int_k;
            } else {  // leaves of the binary build hold at most two primitives
                nd.leafmask |= (uint8_t)(1u << sl);
                if (c->count == 2) nd.twomask |= (uint8_t)(1u << sl);
                for (uint32_t t = 0; t < c->count; ++t) emit_prim(p, refs[c->first + t].id, &out->leaf_prims);
            }
        }
        if (out->nodes.size() < queue.size()) out->nodes.resize(queue.size());
        out->nodes[idx] = nd;
    }
    out->nodes.resize(queue.size());
}

}  // namespace bg
