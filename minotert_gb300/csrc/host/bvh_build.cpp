// Host BVH builder: binned-SAH BVH2 collapsed to the 8-wide quantised node
// format of mrt_cuda.h.  The reference has no acceleration structure (its
// shaders loop over 5 spheres, primaryRay.comp:26-32, secondaryRays.comp:
// 77-83); this module is new and follows published methods:
//   - binned SAH construction (Wald, "On fast construction of SAH-based
//     bounding volume hierarchies", RT 2007), 64 bins per axis;
//   - collapse to 8-wide nodes by the SAH-optimal dynamic programme of
//     Ylitie, Karras & Laine, "Efficient incoherent ray traversal on GPUs
//     through compressed wide BVHs", HPG 2017 (for every BVH2 subtree and
//     every slot budget 1..8, the cheapest way to represent it as one leaf,
//     one 8-wide node or a forest over the budget), or greedily by opening
//     the child of largest surface area; leaves of <= 3 triangles, <= 24 per
//     node, octant-ordered child slots with 8-bit quantised boxes (same
//     paper).
// Quantised boxes are conservative by construction: every child box is
// rounded outward and widened by one quantum when it lands on the grid, so
// a zero-thickness child (a flat triangle, a box face) still has a slab of
// two quanta; traversal adds a relative epsilon on top.
#include "mrt_host.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <future>
#include <memory>
#include <thread>
#include <vector>

namespace {

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const Box& b) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
    }
    void grow(const float* p) {
        for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
    }
    double area() const {
        double d[3];
        for (int a = 0; a < 3; ++a) d[a] = std::max(0.0, double(hi[a]) - double(lo[a]));
        return 2.0 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
    bool valid() const { return lo[0] <= hi[0]; }
};

struct Node2 {
    Box box;
    uint32_t left = 0, right = 0; // children (internal)
    uint32_t first = 0, count = 0; // leaf range in ids (count > 0: leaf)
    uint32_t tris = 0;             // triangles in subtree
};

struct Builder2 {
    const float* verts;
    uint32_t n;
    uint32_t bins;
    uint32_t max_leaf;
    double trav_cost = 0.5;  // SAH cost of a node step / cost of a triangle test
    std::vector<Box> pbox;
    std::vector<float> cent; // 3 per prim
    std::vector<uint32_t> ids;
    std::vector<Node2> nodes;
    std::atomic<uint32_t> next{0};
    int par_depth = 0;

    uint32_t alloc() { return next.fetch_add(1); }

    void build(uint32_t ni, uint32_t begin, uint32_t end, int depth) {
        Node2& node = nodes[ni];
        Box box, cb;
        for (uint32_t i = begin; i < end; ++i) {
            box.grow(pbox[ids[i]]);
            cb.grow(&cent[3 * ids[i]]);
        }
        node.box = box;
        uint32_t cnt = end - begin;
        node.tris = cnt;
        if (cnt == 1) { node.first = begin; node.count = 1; return; }

        // binned SAH over the centroid bounds
        int best_axis = -1;
        uint32_t best_split = 0;
        double best_cost = INFINITY;
        const uint32_t B = bins;
        std::vector<Box> bbox(B);
        std::vector<uint32_t> bcnt(B);
        std::vector<double> rarea(B);
        std::vector<uint32_t> rcnt(B);
        for (int a = 0; a < 3; ++a) {
            double ext = double(cb.hi[a]) - double(cb.lo[a]);
            if (!(ext > 0.0)) continue;
            double scale = double(B) / ext;
            std::fill(bbox.begin(), bbox.end(), Box());
            std::fill(bcnt.begin(), bcnt.end(), 0u);
            for (uint32_t i = begin; i < end; ++i) {
                uint32_t p = ids[i];
                int b = int((double(cent[3 * p + a]) - double(cb.lo[a])) * scale);
                b = std::min(std::max(b, 0), int(B) - 1);
                bbox[b].grow(pbox[p]);
                bcnt[b]++;
            }
            Box acc;
            uint32_t c = 0;
            for (int b = int(B) - 1; b > 0; --b) {
                acc.grow(bbox[b]);
                c += bcnt[b];
                rarea[b] = acc.valid() ? acc.area() : 0.0;
                rcnt[b] = c;
            }
            acc = Box();
            c = 0;
            for (uint32_t b = 0; b + 1 < B; ++b) {
                acc.grow(bbox[b]);
                c += bcnt[b];
                if (c == 0 || rcnt[b + 1] == 0) continue;
                double cost = (acc.valid() ? acc.area() : 0.0) * c + rarea[b + 1] * rcnt[b + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = a; best_split = b + 1; }
            }
        }
        double parea = box.area();
        if (cnt <= max_leaf) {
            // SAH: traversal cost trav_cost, intersection cost 1 (relative to parent area)
            double leaf_cost = double(cnt);
            double split_cost = parea > 0.0 ? trav_cost + best_cost / parea : INFINITY;
            if (best_axis < 0 || leaf_cost <= split_cost) { node.first = begin; node.count = cnt; return; }
        }
        uint32_t mid;
        if (best_axis < 0 || depth > 96) {
            // coincident centroids (or a pathologically deep branch): split
            // by index so the tree stays balanced
            mid = begin + cnt / 2;
        } else {
            const int a = best_axis;
            const double scale = double(bins) / (double(cb.hi[a]) - double(cb.lo[a]));
            const double lo = double(cb.lo[a]);
            auto it = std::partition(ids.begin() + begin, ids.begin() + end, [&](uint32_t p) {
                int b = int((double(cent[3 * p + a]) - lo) * scale);
                b = std::min(std::max(b, 0), int(bins) - 1);
                return uint32_t(b) < best_split;
            });
            mid = uint32_t(it - ids.begin());
            if (mid == begin || mid == end) mid = begin + cnt / 2;
        }
        uint32_t l = alloc(), r = alloc();
        node.left = l;
        node.right = r;
        if (depth < par_depth && cnt > 32768) {
            auto fut = std::async(std::launch::async, [this, l, begin, mid, depth] { build(l, begin, mid, depth + 1); });
            build(r, mid, end, depth + 1);
            fut.get();
        } else {
            build(l, begin, mid, depth + 1);
            build(r, mid, end, depth + 1);
        }
    }
};

// SAH-optimal collapse (Ylitie et al. 2017, section 3.2).  cost[x][i] is
// the least SAH cost of representing BVH2 subtree x by at most i child
// slots of an 8-wide node: one slot (x as a leaf of <= 3 triangles, cost
// area * tris * c_prim, or as an 8-wide node, cost area * c_node plus the
// best distribution of its two children over 8 slots), or, for i >= 2, its
// two children sharing the i slots.  Costs are relative (areas are not
// divided by the root's).
struct CollapseDP {
    struct Entry {
        float cost[9];     // [1..8]
        int8_t split[9];   // [2..8]: slots of the left child when x is opened over i slots (0: x is one slot)
        int8_t dsplit[9];  // [2..8]: the best left/right share when x is opened over i slots
        bool leaf;         // as one slot: a leaf (else an 8-wide node)
    };
    const std::vector<Node2>& n2;
    double c_node, c_prim;
    std::vector<Entry> e;

    CollapseDP(const std::vector<Node2>& nodes, size_t count, double cn, double cp)
        : n2(nodes), c_node(cn), c_prim(cp), e(count) {}

    void solve(uint32_t x) {
        const Node2& n = n2[x];
        Entry& E = e[x];
        const double A = n.box.area();
        if (n.count) {  // a BVH2 leaf is always one leaf slot
            E.leaf = true;
            for (int i = 1; i <= 8; ++i) {
                E.cost[i] = float(A * double(n.count) * c_prim);
                E.split[i] = 0;
                E.dsplit[i] = 0;
            }
            return;
        }
        solve(n.left);
        solve(n.right);
        const Entry& L = e[n.left];
        const Entry& R = e[n.right];
        double dist[9];
        for (int j = 2; j <= 8; ++j) {
            double best = INFINITY;
            int bk = 1;
            for (int k = 1; k < j; ++k) {
                const double c = double(L.cost[k]) + double(R.cost[j - k]);
                if (c < best) { best = c; bk = k; }
            }
            dist[j] = best;
            E.dsplit[j] = int8_t(bk);
        }
        const double as_node = A * c_node + dist[8];
        const double as_leaf = n.tris <= 3 ? A * double(n.tris) * c_prim : INFINITY;
        E.leaf = as_leaf <= as_node;
        E.cost[1] = float(std::min(as_leaf, as_node));
        for (int i = 2; i <= 8; ++i) {
            if (dist[i] < double(E.cost[1])) {
                E.cost[i] = float(dist[i]);
                E.split[i] = E.dsplit[i];
            } else {
                E.cost[i] = E.cost[1];
                E.split[i] = 0;
            }
        }
    }

    // the slots of subtree x under a budget of i
    void slots(uint32_t x, int i, std::vector<uint32_t>& out) const {
        const Entry& E = e[x];
        if (i <= 1 || E.split[i] == 0) { out.push_back(x); return; }
        slots(n2[x].left, E.split[i], out);
        slots(n2[x].right, i - E.split[i], out);
    }
    // the children of x made an 8-wide node
    void children(uint32_t x, std::vector<uint32_t>& out) const {
        const Entry& E = e[x];
        slots(n2[x].left, E.dsplit[8], out);
        slots(n2[x].right, 8 - E.dsplit[8], out);
    }
};

struct Collapser {
    const Builder2& b2;
    const float* verts;
    const CollapseDP* dp = nullptr;  // null: greedy collapse
    std::vector<mrt_bvh8_node> nodes;
    std::vector<mrt_tri> tris;
    uint32_t max_depth = 0;
    uint32_t leaves = 0;
    double sah = 0.0;
    double root_area = 1.0;

    explicit Collapser(const Builder2& b, const float* v) : b2(b), verts(v) {}

    // a child slot holding subtree c2 is a leaf (else an 8-wide node)
    bool is_leaf(uint32_t c2) const {
        const Node2& c = b2.nodes[c2];
        if (c.count) return true;
        return dp ? dp->e[c2].leaf : c.tris <= 3;
    }

    void collect_tris(uint32_t ni, std::vector<uint32_t>& out) const {
        const Node2& n = b2.nodes[ni];
        if (n.count) {
            for (uint32_t i = 0; i < n.count; ++i) out.push_back(b2.ids[n.first + i]);
            return;
        }
        collect_tris(n.left, out);
        collect_tris(n.right, out);
    }

    static void quantize_axis(float lo, float hi, float& origin, int8_t& e_out, double& q) {
        // smallest e with (hi - origin) / 2^e <= 254 where origin <= lo - 2^e
        double ext = double(hi) - double(lo);
        int e = ext > 0.0 ? int(std::ceil(std::log2(ext / 253.0))) - 1 : -100;
        e = std::max(e, -100);
        for (;; ++e) {
            double qv = std::ldexp(1.0, e);
            double o = double(lo) - qv;
            float of = float(o);
            if (double(of) > o) of = std::nextafter(of, -INFINITY);
            if ((double(hi) - double(of)) / qv <= 254.0 || e >= 100) {
                origin = of;
                e_out = int8_t(e);
                q = qv;
                return;
            }
        }
    }

    void emit(uint32_t slot_index, uint32_t root2, uint32_t depth) {
        max_depth = std::max(max_depth, depth);
        const Node2& r = b2.nodes[root2];
        // 1) gather up to 8 child subtrees by opening the largest ones
        std::vector<uint32_t> cand;
        if (r.count) cand.push_back(root2);
        else if (dp) dp->children(root2, cand);
        else { cand.push_back(r.left); cand.push_back(r.right); }
        for (int pass = 0; pass < 2 && !dp; ++pass) {
            while (cand.size() < 8) {
                int pick = -1;
                double best = -1.0;
                for (size_t i = 0; i < cand.size(); ++i) {
                    const Node2& c = b2.nodes[cand[i]];
                    if (c.count) continue;              // BVH2 leaf
                    if (pass == 0 && c.tris <= 3) continue; // pass 0: must-open
                    double a = c.box.area();
                    if (a > best) { best = a; pick = int(i); }
                }
                if (pick < 0) break;
                uint32_t o = cand[pick];
                cand[pick] = b2.nodes[o].left;
                cand.push_back(b2.nodes[o].right);
            }
        }
        const int nc = int(cand.size());
        // 2) octant slot assignment (greedy over cost = dot(c - p, d_slot))
        Box pbox;
        for (uint32_t c : cand) pbox.grow(b2.nodes[c].box);
        double pc[3], cc[8][3];
        for (int a = 0; a < 3; ++a) pc[a] = 0.5 * (double(pbox.lo[a]) + double(pbox.hi[a]));
        for (int i = 0; i < nc; ++i)
            for (int a = 0; a < 3; ++a)
                cc[i][a] = 0.5 * (double(b2.nodes[cand[i]].box.lo[a]) + double(b2.nodes[cand[i]].box.hi[a])) - pc[a];
        int slot_of[8];
        bool used_slot[8] = {}, used_c[8] = {};
        for (int k = 0; k < nc; ++k) {
            double best = INFINITY;
            int bi = -1, bs = -1;
            for (int i = 0; i < nc; ++i) {
                if (used_c[i]) continue;
                for (int s = 0; s < 8; ++s) {
                    if (used_slot[s]) continue;
                    double d = cc[i][0] * ((s & 1) ? -1.0 : 1.0) + cc[i][1] * ((s & 2) ? -1.0 : 1.0) +
                               cc[i][2] * ((s & 4) ? -1.0 : 1.0);
                    if (d < best) { best = d; bi = i; bs = s; }
                }
            }
            used_c[bi] = true;
            used_slot[bs] = true;
            slot_of[bi] = bs;
        }
        int child_at[8];
        for (int s = 0; s < 8; ++s) child_at[s] = -1;
        for (int i = 0; i < nc; ++i) child_at[slot_of[i]] = i;

        // 3) node header and quantisation
        mrt_bvh8_node nd;
        std::memset(&nd, 0, sizeof(nd));
        double qs[3];
        for (int a = 0; a < 3; ++a) quantize_axis(pbox.lo[a], pbox.hi[a], nd.origin[a], nd.exp[a], qs[a]);
        uint8_t* qlo[3] = {nd.q_lo_x, nd.q_lo_y, nd.q_lo_z};
        uint8_t* qhi[3] = {nd.q_hi_x, nd.q_hi_y, nd.q_hi_z};

        // internal children get a contiguous block in slot order
        uint32_t n_int = 0;
        for (int s = 0; s < 8; ++s)
            if (child_at[s] >= 0 && !is_leaf(cand[child_at[s]])) n_int++;
        uint32_t child_base = uint32_t(nodes.size());
        nodes.resize(nodes.size() + n_int);
        nd.child_base = child_base;
        nd.tri_base = uint32_t(tris.size());
        std::vector<std::pair<uint32_t, uint32_t>> recurse; // (node8 index, node2)
        uint32_t k_int = 0, tri_off = 0;
        for (int s = 0; s < 8; ++s) {
            if (child_at[s] < 0) continue;
            uint32_t c2 = cand[child_at[s]];
            const Node2& c = b2.nodes[c2];
            for (int a = 0; a < 3; ++a) {
                double lo = (double(c.box.lo[a]) - double(nd.origin[a])) / qs[a];
                double hi = (double(c.box.hi[a]) - double(nd.origin[a])) / qs[a];
                double fl = std::floor(lo), ch = std::ceil(hi);
                if (fl == lo) fl -= 1.0;
                if (ch == hi) ch += 1.0;
                fl = std::max(0.0, fl);
                ch = std::min(255.0, ch);
                qlo[a][s] = uint8_t(fl);
                qhi[a][s] = uint8_t(ch);
            }
            if (!is_leaf(c2)) {
                nd.imask |= uint8_t(1u << s);
                nd.meta[s] = uint8_t(0x20 | (24 + s));
                recurse.push_back({child_base + k_int, c2});
                k_int++;
                sah += c.box.area() / root_area * 1.0;
            } else {
                std::vector<uint32_t> ts;
                collect_tris(c2, ts);
                uint32_t k = uint32_t(ts.size());
                nd.meta[s] = uint8_t((((1u << k) - 1u) << 5) | tri_off);
                for (uint32_t t : ts) {
                    mrt_tri tr;
                    const float* v = verts + 9ull * t;
                    tr.v0[0] = v[0]; tr.v0[1] = v[1]; tr.v0[2] = v[2]; tr.id = t;
                    tr.v1[0] = v[3]; tr.v1[1] = v[4]; tr.v1[2] = v[5]; tr.pad1 = 0;
                    tr.v2[0] = v[6]; tr.v2[1] = v[7]; tr.v2[2] = v[8]; tr.pad2 = 0;
                    tris.push_back(tr);
                }
                tri_off += k;
                leaves++;
                sah += c.box.area() / root_area * double(k) * 0.3;
            }
        }
        nodes[slot_index] = nd;
        for (auto& rc : recurse) emit(rc.first, rc.second, depth + 1);
    }
};

} // namespace

extern "C" {

void mrt_bvh8_free(mrt_bvh8* bvh) {
    if (!bvh) return;
    std::free(bvh->nodes);
    std::free(bvh->tris);
    bvh->nodes = nullptr;
    bvh->tris = nullptr;
    bvh->node_count = bvh->tri_count = 0;
}

int mrt_bvh8_build(const float* verts, uint32_t tri_count, const mrt_bvh_build_params* params,
                   mrt_bvh8* out) {
    if (!verts || !out || tri_count == 0) return MRT_EINVAL;
    std::memset(out, 0, sizeof(*out));
    auto t0 = std::chrono::steady_clock::now();
    Builder2 b;
    b.verts = verts;
    b.n = tri_count;
    b.bins = params && params->sah_bins ? params->sah_bins : 64;
    b.trav_cost = params && params->trav_cost_pct ? double(params->trav_cost_pct) / 100.0 : 0.5;
    b.max_leaf = params && params->max_leaf_tris ? std::min<uint32_t>(params->max_leaf_tris, 3) : 3;
    b.bins = std::max<uint32_t>(4, std::min<uint32_t>(b.bins, 256));
    unsigned threads = params && params->threads ? params->threads : std::thread::hardware_concurrency();
    threads = std::max(1u, threads);
    b.par_depth = 0;
    while ((1u << b.par_depth) < threads * 2 && b.par_depth < 12) b.par_depth++;
    b.pbox.resize(tri_count);
    b.cent.resize(3ull * tri_count);
    b.ids.resize(tri_count);
    for (uint32_t i = 0; i < tri_count; ++i) {
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(verts[9ull * i + k])) return MRT_EINVAL;
        Box bx;
        for (int k = 0; k < 3; ++k) bx.grow(verts + 9ull * i + 3 * k);
        for (int a = 0; a < 3; ++a) {
            if (!std::isfinite(bx.lo[a]) || !std::isfinite(bx.hi[a])) return MRT_EINVAL;
            b.cent[3ull * i + a] = 0.5f * bx.lo[a] + 0.5f * bx.hi[a];
        }
        b.pbox[i] = bx;
        b.ids[i] = i;
    }
    b.nodes.resize(2ull * tri_count);
    uint32_t root = b.alloc();
    b.build(root, 0, tri_count, 0);

    Collapser c(b, verts);
    c.root_area = std::max(1e-30, b.nodes[root].box.area());
    std::unique_ptr<CollapseDP> dp;
    if (params && params->collapse == 1) {
        const double cp = params && params->prim_cost_pct ? double(params->prim_cost_pct) / 100.0 : 0.3;
        dp.reset(new CollapseDP(b.nodes, b.next.load(), 1.0, cp));
        dp->solve(root);
        c.dp = dp.get();
    }
    c.nodes.reserve(tri_count / 3 + 16);
    c.tris.reserve(tri_count);
    c.nodes.resize(1);
    c.emit(0, root, 1);

    out->node_count = uint32_t(c.nodes.size());
    out->tri_count = uint32_t(c.tris.size());
    out->nodes = static_cast<mrt_bvh8_node*>(std::aligned_alloc(128, sizeof(mrt_bvh8_node) * c.nodes.size()));
    out->tris = static_cast<mrt_tri*>(std::malloc(sizeof(mrt_tri) * c.tris.size()));
    if (!out->nodes || !out->tris) {
        mrt_bvh8_free(out);
        return MRT_ENOMEM;
    }
    std::memcpy(out->nodes, c.nodes.data(), sizeof(mrt_bvh8_node) * c.nodes.size());
    std::memcpy(out->tris, c.tris.data(), sizeof(mrt_tri) * c.tris.size());
    out->depth = c.max_depth;
    out->leaf_count = c.leaves;
    out->sah_cost = c.sah;
    out->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return MRT_OK;
}

} // extern "C"
