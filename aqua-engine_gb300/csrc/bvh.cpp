// bvh.cpp — binned-SAH build (32 bins x 3 axes), subtrees above 64K
// triangles built on separate threads, flattened depth-first.
#include "bvh.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cfloat>
#include <cstring>
#include <future>
#include <limits>
#include <thread>

namespace aq {
namespace {

struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    bool empty() const { return lo[0] > hi[0]; }
    double area() const {
        if (empty()) return 0.0;
        double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct BNode {
    Box box;
    int left = -1, right = -1;  // children (indices in the same vector) when inner
    int first = 0, count = 0;   // prim range when leaf
    bool leaf() const { return left < 0; }
};

struct Ctx {
    const std::vector<Box>* boxes;
    const std::vector<float>* cent;  // 3 per prim
    std::vector<int32_t>* refs;
    std::atomic<int> threads{1};
    int max_threads = 1;
};

constexpr int kBins = 32;
constexpr size_t kParallelMin = 65536;

// Builds the subtree over refs[begin, end) into out; returns its root index.
int build_rec(Ctx& C, std::vector<BNode>& out, int begin, int end, int depth) {
    const auto& boxes = *C.boxes;
    const auto& cent = *C.cent;
    auto& refs = *C.refs;
    int node = (int)out.size();
    out.emplace_back();
    Box bb, cb;
    for (int i = begin; i < end; ++i) {
        bb.grow(boxes[(size_t)refs[(size_t)i]]);
        cb.grow(&cent[3 * (size_t)refs[(size_t)i]]);
    }
    out[(size_t)node].box = bb;
    int n = end - begin;
    auto make_leaf = [&]() {
        out[(size_t)node].first = begin;
        out[(size_t)node].count = n;
        return node;
    };
    if (n <= 1) return make_leaf();

    // Binned SAH over the three axes.
    double best_cost = DBL_MAX;
    int best_axis = -1, best_split = -1;
    if (depth < 32) {
        for (int ax = 0; ax < 3; ++ax) {
            float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.0f)) continue;
            float k = (float)kBins * (1.0f - 1e-6f) / ext;
            Box bbox[kBins];
            int bcnt[kBins] = {0};
            for (int i = begin; i < end; ++i) {
                int p = refs[(size_t)i];
                int b = (int)((cent[3 * (size_t)p + ax] - cb.lo[ax]) * k);
                b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                bcnt[b]++;
                bbox[b].grow(boxes[(size_t)p]);
            }
            double rarea[kBins];
            int rcnt[kBins];
            Box acc;
            int c = 0;
            for (int b = kBins - 1; b > 0; --b) {
                acc.grow(bbox[b]);
                c += bcnt[b];
                rarea[b] = acc.area();
                rcnt[b] = c;
            }
            Box lacc;
            int lc = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                lacc.grow(bbox[b]);
                lc += bcnt[b];
                if (lc == 0 || rcnt[b + 1] == 0) continue;
                double cost = lacc.area() * lc + rarea[b + 1] * rcnt[b + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = ax;
                    best_split = b + 1;
                }
            }
        }
    }
    double parea = bb.area();
    double split_cost = best_axis >= 0 ? 1.0 + best_cost / std::max(parea, 1e-30) : DBL_MAX;
    if (n <= kBvhMaxLeaf && (double)n <= split_cost) return make_leaf();

    int mid;
    if (best_axis >= 0) {
        float ext = cb.hi[best_axis] - cb.lo[best_axis];
        float k = (float)kBins * (1.0f - 1e-6f) / ext;
        int ax = best_axis;
        auto it = std::partition(refs.begin() + begin, refs.begin() + end, [&](int32_t p) {
            int b = (int)((cent[3 * (size_t)p + ax] - cb.lo[ax]) * k);
            b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
            return b < best_split;
        });
        mid = (int)(it - refs.begin());
    } else {
        // Degenerate centroids or deep tree: median split on the widest axis.
        int ax = 0;
        for (int k = 1; k < 3; ++k)
            if (cb.hi[k] - cb.lo[k] > cb.hi[ax] - cb.lo[ax]) ax = k;
        mid = begin + n / 2;
        std::nth_element(refs.begin() + begin, refs.begin() + mid, refs.begin() + end,
                         [&](int32_t a, int32_t b) {
                             float ca = cent[3 * (size_t)a + ax], cbv = cent[3 * (size_t)b + ax];
                             return ca < cbv || (ca == cbv && a < b);
                         });
    }
    if (mid == begin || mid == end) mid = begin + n / 2;

    int left, right;
    if ((size_t)n >= kParallelMin && C.threads.fetch_add(1) < C.max_threads) {
        std::vector<BNode> lsub;
        auto fut = std::async(std::launch::async, [&]() { build_rec(C, lsub, begin, mid, depth + 1); });
        std::vector<BNode> rsub;
        build_rec(C, rsub, mid, end, depth + 1);
        fut.get();
        C.threads.fetch_sub(1);
        // Merge: left subtree first, then right, indices shifted.
        left = (int)out.size();
        for (auto nd : lsub) {
            if (!nd.leaf()) { nd.left += left; nd.right += left; }
            out.push_back(nd);
        }
        right = (int)out.size();
        for (auto nd : rsub) {
            if (!nd.leaf()) { nd.left += right; nd.right += right; }
            out.push_back(nd);
        }
    } else {
        if ((size_t)n >= kParallelMin) C.threads.fetch_sub(1);
        left = build_rec(C, out, begin, mid, depth + 1);
        right = build_rec(C, out, mid, end, depth + 1);
    }
    out[(size_t)node].left = left;
    out[(size_t)node].right = right;
    return node;
}

}  // namespace

FlatBvh build_bvh(const float* verts, size_t num_tris) {
    std::vector<Box> boxes(num_tris);
    std::vector<float> cent(3 * num_tris);
    for (size_t i = 0; i < num_tris; ++i) {
        for (int c = 0; c < 3; ++c) boxes[i].grow(&verts[9 * i + 3 * (size_t)c]);
        for (int k = 0; k < 3; ++k) cent[3 * i + (size_t)k] = 0.5f * boxes[i].lo[k] + 0.5f * boxes[i].hi[k];
    }
    std::vector<int32_t> refs(num_tris);
    for (size_t i = 0; i < num_tris; ++i) refs[i] = (int32_t)i;

    std::vector<BNode> tree;
    tree.reserve(num_tris > 0 ? 2 * num_tris : 1);
    Ctx C;
    C.boxes = &boxes;
    C.cent = &cent;
    C.refs = &refs;
    C.max_threads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (num_tris > 0) build_rec(C, tree, 0, (int)num_tris, 0);

    FlatBvh out;
    // Root as a two-child inner node even when the tree is a single leaf.
    if (num_tris == 0 || tree[0].leaf()) {
        BNode root, a, b;
        if (num_tris > 0) a = tree[0];
        else { float z[3] = {0, 0, 0}; a.box.grow(z); }
        b = a;
        b.count = 0;
        tree.clear();
        root.box = a.box;
        root.left = 1;
        root.right = 2;
        tree.push_back(root);
        tree.push_back(a);
        tree.push_back(b);
    }

    // Collapse into wide nodes, numbered depth first: wide[k] lists the
    // binary nodes that become node k's children, in spatial (left to right)
    // order; an inner child of largest surface area is replaced by its two
    // children while fewer than kBvhWidth are held (ties: the leftmost).
    struct Wide {
        int ch[kBvhWidth];
        int n;
    };
    std::vector<Wide> wide;
    std::vector<int> wid(tree.size(), -1);
    {
        std::vector<int> st{0};
        while (!st.empty()) {
            int b = st.back();
            st.pop_back();
            Wide w;
            w.n = 2;
            w.ch[0] = tree[(size_t)b].left;
            w.ch[1] = tree[(size_t)b].right;
            while (w.n < kBvhWidth) {
                int pick = -1;
                double best = -1.0;
                for (int k = 0; k < w.n; ++k) {
                    const BNode& c = tree[(size_t)w.ch[k]];
                    if (c.leaf()) continue;
                    double a = c.box.area();
                    if (a > best) { best = a; pick = k; }
                }
                if (pick < 0) break;
                int l = tree[(size_t)w.ch[pick]].left, r = tree[(size_t)w.ch[pick]].right;
                for (int k = w.n; k > pick + 1; --k) w.ch[k] = w.ch[k - 1];
                w.ch[pick] = l;
                w.ch[pick + 1] = r;
                ++w.n;
            }
            wid[(size_t)b] = (int)wide.size();
            wide.push_back(w);
            for (int k = w.n - 1; k >= 0; --k)
                if (!tree[(size_t)w.ch[k]].leaf()) st.push_back(w.ch[k]);
        }
    }

    const float inf = std::numeric_limits<float>::infinity();
    out.nodes.assign((size_t)kBvhNodeFloats * wide.size(), 0.0f);
    out.tri_order.reserve(num_tris);
    int max_leaf = 0;
    // Depth of every wide node (root = 1) and the stack entries a ray holds
    // when it arrives there (the other hit children pushed on the way).
    std::vector<int> depth(wide.size(), 0), need(wide.size(), 0);
    depth[0] = 1;
    int max_depth = 1, max_stack = 0;
    for (size_t k = 0; k < wide.size(); ++k) {
        const Wide& wn = wide[k];
        float* w = &out.nodes[(size_t)kBvhNodeFloats * k];
        int32_t link[kBvhWidth], count[kBvhWidth];
        const int pushes = need[k] + wn.n - 1;
        max_stack = std::max(max_stack, pushes);
        for (int c = 0; c < kBvhWidth; ++c) {
            if (c >= wn.n) {
                for (int a = 0; a < 6; ++a) w[4 * a + c] = inf;
                link[c] = ~0;
                count[c] = 0;
                continue;
            }
            const BNode& cn = tree[(size_t)wn.ch[c]];
            for (int a = 0; a < 3; ++a) {
                w[8 * a + c] = cn.box.lo[a];
                w[8 * a + 4 + c] = cn.box.hi[a];
            }
            if (cn.leaf()) {
                int first = (int)out.tri_order.size();
                for (int i = 0; i < cn.count; ++i) out.tri_order.push_back(refs[(size_t)(cn.first + i)]);
                link[c] = ~((first << 3) | cn.count);
                count[c] = cn.count;
                max_leaf = std::max(max_leaf, cn.count);
            } else {
                int ci = wid[(size_t)wn.ch[c]];
                link[c] = ci;
                count[c] = 0;
                depth[(size_t)ci] = depth[k] + 1;
                need[(size_t)ci] = pushes;
                max_depth = std::max(max_depth, depth[(size_t)ci]);
            }
        }
        memcpy(&w[24], link, sizeof(link));
        memcpy(&w[28], count, sizeof(count));
    }
    for (int a = 0; a < 3; ++a) {
        out.lo[a] = tree[0].box.lo[a];
        out.hi[a] = tree[0].box.hi[a];
    }
    out.max_stack = max_stack;
    out.depth = max_depth;
    out.max_leaf = max_leaf;
    return out;
}

// ------------------------------------------------------------------ quantized copy
namespace {
float scale_of(int e) {  // 2^(e - 127), e in [1, 254]
    uint32_t b = (uint32_t)e << 23;
    float f;
    memcpy(&f, &b, 4);
    return f;
}
// The plane a byte decodes to, exactly as the device computes it.
float decode_plane(int q, float s, float o) { return std::fmaf((float)q, s, o); }
}  // namespace

std::vector<float> quantize_bvh(const FlatBvh& bvh) {
    const int nn = bvh.num_nodes();
    std::vector<float> out((size_t)kBvhQNodeFloats * (size_t)nn, 0.0f);
    for (int k = 0; k < nn; ++k) {
        const float* w = &bvh.nodes[(size_t)kBvhNodeFloats * (size_t)k];
        int32_t link[4], count[4];
        memcpy(link, &w[24], 16);
        memcpy(count, &w[28], 16);
        float* q = &out[(size_t)kBvhQNodeFloats * (size_t)k];
        uint32_t bytes[6] = {0, 0, 0, 0, 0, 0};  // qlo.x, qhi.x, qlo.y, qhi.y, qlo.z, qhi.z
        uint32_t exps = 0, counts = 0;
        for (int a = 0; a < 3; ++a) {
            float lo = std::numeric_limits<float>::infinity(), hi = -lo;
            for (int c = 0; c < 4; ++c) {
                if (link[c] == ~0) continue;
                lo = std::min(lo, w[8 * a + c]);
                hi = std::max(hi, w[8 * a + 4 + c]);
            }
            if (!(lo <= hi)) lo = hi = 0.0f;  // no children (not produced by the builder)
            const float o = lo;
            // Smallest power-of-two step whose 255 steps reach the far side,
            // then the next ones while some child's plane does not fit.
            int e = 1;
            while (e < 254 && (double)scale_of(e) * 255.0 < (double)hi - (double)o) ++e;
            for (;; ++e) {
                const float sc = scale_of(e);
                bool fits = true;
                uint32_t blo = 0, bhi = 0;
                for (int c = 0; c < 4 && fits; ++c) {
                    int ql = 255, qh = 0;  // empty slot: skipped by its link
                    if (link[c] != ~0) {
                        const float clo = w[8 * a + c], chi = w[8 * a + 4 + c];
                        ql = (int)std::floor(((double)clo - (double)o) / (double)sc);
                        ql = std::max(0, std::min(255, ql));
                        while (ql > 0 && decode_plane(ql, sc, o) > clo) --ql;
                        qh = (int)std::ceil(((double)chi - (double)o) / (double)sc);
                        qh = std::max(0, qh);
                        while (qh <= 255 && decode_plane(qh, sc, o) < chi) ++qh;
                        if (qh > 255 || decode_plane(ql, sc, o) > clo) fits = false;
                    }
                    blo |= (uint32_t)ql << (8 * c);
                    bhi |= (uint32_t)std::min(qh, 255) << (8 * c);
                }
                if (fits || e >= 254) {
                    bytes[2 * a] = blo;
                    bytes[2 * a + 1] = bhi;
                    exps |= (uint32_t)e << (8 * a);
                    q[a] = o;
                    break;
                }
            }
        }
        for (int c = 0; c < 4; ++c) counts |= (uint32_t)(count[c] & 0xff) << (8 * c);
        memcpy(&q[3], &exps, 4);
        memcpy(&q[4], link, 16);
        memcpy(&q[8], bytes, 16);
        memcpy(&q[12], &bytes[4], 8);
        memcpy(&q[14], &counts, 4);
    }
    return out;
}

}  // namespace aq
