// Spatial-split BVH builder (host): the library's binned SAH builder with spatial splits
// added, after Stich, Friedrich and Dietrich, "Spatial Splits in Bounding Volume
// Hierarchies" (HPG 2009) -- the same idea as the reference's SplitBVH
// (splitbvh.cpp:664-1408), built here in its own way:
//
//  * references (a primitive and its clipped box) are split between the children; a node
//    tries the best object split (32 centroid bins per axis) and, when the two object-split
//    children overlap by more than 1e-5 of the root's surface area, the best spatial split
//    (32 equal bins per axis of the node box, each reference's triangle clipped to the bins
//    it spans); the cheaper one wins (SAH, unit node and triangle costs);
//  * a reference straddling a spatial plane goes to both children with its triangle
//    clipped to each side: the clipped polygon is computed in double precision and its
//    bounds rounded outwards to float, then intersected with the reference's box, so every
//    box contains the part of the triangle it stands for;
//  * spatial splits stop once the references have grown by a third over the triangles, and
//    below a depth of 48 (the traversal stacks hold 62 levels).
// Large subtrees are built in parallel.  Leaves hold at most leaf_size references.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <future>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

#include "host.h"

namespace mcrt {
namespace {

constexpr int    kObjBins = 32;
constexpr int    kSpatialBins = 32;
constexpr double kAlpha = 1e-5;
constexpr int    kMaxSpatialDepth = 48;

struct Box
{
    float lo[3], hi[3];
    Box() { reset(); }
    void reset()
    {
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = std::numeric_limits<float>::infinity();
            hi[k] = -std::numeric_limits<float>::infinity();
        }
    }
    bool empty() const { return !(hi[0] >= lo[0] && hi[1] >= lo[1] && hi[2] >= lo[2]); }
    void grow(const Box& b)
    {
        for (int k = 0; k < 3; ++k)
        {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    double half_area() const
    {
        if (empty()) return 0.0;
        double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
    float centre(int k) const { return 0.5f * (lo[k] + hi[k]); }
};

Box intersect(const Box& a, const Box& b)
{
    Box r;
    for (int k = 0; k < 3; ++k)
    {
        r.lo[k] = std::max(a.lo[k], b.lo[k]);
        r.hi[k] = std::min(a.hi[k], b.hi[k]);
    }
    return r;
}

struct Ref
{
    int32_t prim;
    Box     box;
};

// bounds of the part of triangle `prim` with lo <= x[axis] <= hi, intersected with `clip`
// (empty when the triangle has no part there); the polygon is clipped in double precision
// and its bounds rounded outwards to float
Box clip_triangle(const float* v, int32_t prim, int axis, double lo, double hi, const Box& clip)
{
    double poly[9][3], tmp[9][3];
    int    n = 3;
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) poly[i][k] = v[9 * static_cast<int64_t>(prim) + 3 * i + k];
    for (int side = 0; side < 2; ++side)
    {
        // keep x >= lo (side 0) / x <= hi (side 1)
        auto inside = [&](const double* p) { return side == 0 ? p[axis] >= lo : p[axis] <= hi; };
        const double plane = side == 0 ? lo : hi;
        int          m = 0;
        for (int i = 0; i < n; ++i)
        {
            const double* a = poly[i];
            const double* b = poly[(i + 1) % n];
            const bool    ia = inside(a), ib = inside(b);
            if (ia) std::copy(a, a + 3, tmp[m++]);
            if (ia != ib)
            {
                const double t = (plane - a[axis]) / (b[axis] - a[axis]);
                for (int k = 0; k < 3; ++k) tmp[m][k] = a[k] + t * (b[k] - a[k]);
                tmp[m][axis] = plane;
                ++m;
            }
        }
        n = m;
        for (int i = 0; i < n; ++i) std::copy(tmp[i], tmp[i] + 3, poly[i]);
        if (n == 0) return Box();
    }
    Box r;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k)
        {
            float f = static_cast<float>(poly[i][k]);
            float down = static_cast<double>(f) > poly[i][k] ? std::nextafter(f, -INFINITY) : f;
            float up = static_cast<double>(f) < poly[i][k] ? std::nextafter(f, INFINITY) : f;
            r.lo[k] = std::min(r.lo[k], down);
            r.hi[k] = std::max(r.hi[k], up);
        }
    return intersect(r, clip);
}

struct SplitBuilder
{
    const float*          v;
    int                   leaf_size;
    double                alpha_area = 0.0;
    int64_t               ref_budget = 0;
    std::atomic<int64_t>  extra_refs{0};
    std::atomic<int>      threads_left{0};
    std::mutex            mu;
    std::vector<Box>      nbox;
    std::vector<int32_t>  ninfo;
    std::vector<Ref>      leaf_refs;

    int new_node()
    {
        std::lock_guard<std::mutex> lock(mu);
        nbox.emplace_back();
        ninfo.resize(ninfo.size() + 6, 0);
        return static_cast<int>(nbox.size()) - 1;
    }

    void set_node(int node, const Box& b, const int32_t (&info)[6])
    {
        std::lock_guard<std::mutex> lock(mu);
        nbox[node] = b;
        std::copy(info, info + 6, &ninfo[6 * static_cast<size_t>(node)]);
    }

    void make_leaf(int node, const Box& bb, const std::vector<Ref>& refs)
    {
        int32_t begin;
        {
            std::lock_guard<std::mutex> lock(mu);
            begin = static_cast<int32_t>(leaf_refs.size());
            leaf_refs.insert(leaf_refs.end(), refs.begin(), refs.end());
        }
        const int32_t info[6] = {1, -1, -1, 0, begin, static_cast<int32_t>(refs.size())};
        set_node(node, bb, info);
    }

    struct ObjectSplit
    {
        double cost = std::numeric_limits<double>::infinity();
        int    axis = -1, bin = -1;
        Box    left, right;
        float  lo = 0.f, scale = 0.f;
    };

    ObjectSplit best_object(const std::vector<Ref>& refs) const
    {
        Box cb;
        for (const Ref& r : refs)
            for (int k = 0; k < 3; ++k)
            {
                cb.lo[k] = std::min(cb.lo[k], r.box.centre(k));
                cb.hi[k] = std::max(cb.hi[k], r.box.centre(k));
            }
        ObjectSplit best;
        for (int ax = 0; ax < 3; ++ax)
        {
            const float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.f)) continue;
            const float scale = kObjBins / ext;
            Box         bin_box[kObjBins];
            int         bin_cnt[kObjBins] = {0};
            for (const Ref& r : refs)
            {
                const int b = std::min(kObjBins - 1, static_cast<int>((r.box.centre(ax) - cb.lo[ax]) * scale));
                bin_cnt[b]++;
                bin_box[b].grow(r.box);
            }
            Box    right_box[kObjBins];
            int    right_cnt[kObjBins];
            Box    acc;
            int    c = 0;
            for (int b = kObjBins - 1; b > 0; --b)
            {
                acc.grow(bin_box[b]);
                c += bin_cnt[b];
                right_box[b] = acc;
                right_cnt[b] = c;
            }
            acc.reset();
            c = 0;
            for (int b = 0; b < kObjBins - 1; ++b)
            {
                acc.grow(bin_box[b]);
                c += bin_cnt[b];
                if (c == 0 || right_cnt[b + 1] == 0) continue;
                const double cost = acc.half_area() * c + right_box[b + 1].half_area() * right_cnt[b + 1];
                if (cost < best.cost)
                {
                    best.cost = cost;
                    best.axis = ax;
                    best.bin = b;
                    best.left = acc;
                    best.right = right_box[b + 1];
                    best.lo = cb.lo[ax];
                    best.scale = scale;
                }
            }
        }
        return best;
    }

    struct SpatialSplit
    {
        double cost = std::numeric_limits<double>::infinity();
        int    axis = -1;
        float  plane = 0.f;
    };

    SpatialSplit best_spatial(const std::vector<Ref>& refs, const Box& bb) const
    {
        SpatialSplit best;
        for (int ax = 0; ax < 3; ++ax)
        {
            const double lo = bb.lo[ax], hi = bb.hi[ax];
            if (!(hi > lo)) continue;
            const double width = (hi - lo) / kSpatialBins;
            Box          bin_box[kSpatialBins];
            int          entry[kSpatialBins] = {0}, exit[kSpatialBins] = {0};
            auto         bin_of = [&](double x) {
                return std::max(0, std::min(kSpatialBins - 1, static_cast<int>((x - lo) / width)));
            };
            for (const Ref& r : refs)
            {
                const int b0 = bin_of(r.box.lo[ax]), b1 = bin_of(r.box.hi[ax]);
                entry[b0]++;
                exit[b1]++;
                if (b0 == b1)
                {
                    bin_box[b0].grow(r.box);
                    continue;
                }
                for (int b = b0; b <= b1; ++b)
                {
                    const Box part = clip_triangle(v, r.prim, ax, lo + b * width, lo + (b + 1) * width, r.box);
                    if (!part.empty()) bin_box[b].grow(part);
                }
            }
            Box right_box[kSpatialBins];
            int right_cnt[kSpatialBins];
            Box acc;
            int c = 0;
            for (int b = kSpatialBins - 1; b > 0; --b)
            {
                acc.grow(bin_box[b]);
                c += exit[b];
                right_box[b] = acc;
                right_cnt[b] = c;
            }
            acc.reset();
            c = 0;
            for (int b = 0; b < kSpatialBins - 1; ++b)
            {
                acc.grow(bin_box[b]);
                c += entry[b];
                if (c == 0 || right_cnt[b + 1] == 0) continue;
                const double cost = acc.half_area() * c + right_box[b + 1].half_area() * right_cnt[b + 1];
                if (cost < best.cost)
                {
                    best.cost = cost;
                    best.axis = ax;
                    best.plane = static_cast<float>(lo + (b + 1) * width);
                }
            }
        }
        return best;
    }

    void build(int node, std::vector<Ref> refs, int depth)
    {
        Box bb;
        for (const Ref& r : refs) bb.grow(r.box);
        const size_t count = refs.size();
        if (count <= static_cast<size_t>(leaf_size))
        {
            make_leaf(node, bb, refs);
            return;
        }
        ObjectSplit  os = best_object(refs);
        SpatialSplit ss;
        if (depth < kMaxSpatialDepth && extra_refs.load() < ref_budget && os.axis >= 0)
        {
            const Box overlap = intersect(os.left, os.right);
            if (!overlap.empty() && overlap.half_area() > alpha_area) ss = best_spatial(refs, bb);
        }
        std::vector<Ref> left, right;
        int              axis = 0;
        if (ss.axis >= 0 && ss.cost < os.cost)
        {
            axis = ss.axis;
            const float p = ss.plane;
            for (const Ref& r : refs)
            {
                if (r.box.hi[axis] <= p)
                    left.push_back(r);
                else if (r.box.lo[axis] >= p)
                    right.push_back(r);
                else
                {
                    const double inf = std::numeric_limits<double>::infinity();
                    const Box    lb = clip_triangle(v, r.prim, axis, -inf, p, r.box);
                    const Box    rb = clip_triangle(v, r.prim, axis, p, inf, r.box);
                    if (!lb.empty()) left.push_back(Ref{r.prim, lb});
                    if (!rb.empty()) right.push_back(Ref{r.prim, rb});
                }
            }
            const int64_t grown = static_cast<int64_t>(left.size() + right.size()) - static_cast<int64_t>(count);
            if (grown > 0) extra_refs.fetch_add(grown);
            if (left.empty() || right.empty())  // degenerate: fall back to the object split
            {
                left.clear();
                right.clear();
                ss.axis = -1;
            }
        }
        if (left.empty() && right.empty())
        {
            if (os.axis >= 0)
            {
                axis = os.axis;
                for (const Ref& r : refs)
                {
                    const int b =
                        std::min(kObjBins - 1, static_cast<int>((r.box.centre(os.axis) - os.lo) * os.scale));
                    (b <= os.bin ? left : right).push_back(r);
                }
            }
            if (left.empty() || right.empty())  // coincident centroids: halves
            {
                left.assign(refs.begin(), refs.begin() + count / 2);
                right.assign(refs.begin() + count / 2, refs.end());
            }
        }
        refs.clear();
        refs.shrink_to_fit();
        const int     l = new_node(), r = new_node();
        const int32_t info[6] = {0, l, r, axis, 0, 0};
        set_node(node, bb, info);
        if (count > 16384 && threads_left.fetch_sub(1) > 0)
        {
            auto fut = std::async(std::launch::async,
                                  [this, l, depth, lv = std::move(left)]() mutable { build(l, std::move(lv), depth + 1); });
            build(r, std::move(right), depth + 1);
            fut.get();
        }
        else
        {
            build(l, std::move(left), depth + 1);
            build(r, std::move(right), depth + 1);
        }
    }
};

}  // namespace

void build_split_tree(const float* v, int64_t n, int leaf_size, BinaryTree& out)
{
    if (leaf_size <= 0) leaf_size = kDefaultLeafSize;
    SplitBuilder b;
    b.v = v;
    b.leaf_size = leaf_size;
    std::vector<Ref> refs(static_cast<size_t>(n));
    Box              root;
    for (int64_t i = 0; i < n; ++i)
    {
        Ref& r = refs[i];
        r.prim = static_cast<int32_t>(i);
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k)
            {
                const float x = v[9 * i + 3 * c + k];
                r.box.lo[k] = std::min(r.box.lo[k], x);
                r.box.hi[k] = std::max(r.box.hi[k], x);
            }
        root.grow(r.box);
    }
    b.alpha_area = kAlpha * root.half_area();
    b.ref_budget = n / 3;
    unsigned hw = std::thread::hardware_concurrency();
    b.threads_left = static_cast<int>(hw ? 2 * hw : 8);
    const int root_node = b.new_node();
    b.build(root_node, std::move(refs), 0);
    const size_t nn = b.nbox.size();
    out.node_box.resize(6 * nn);
    out.node_info = b.ninfo;
    for (size_t i = 0; i < nn; ++i)
        for (int k = 0; k < 3; ++k)
        {
            out.node_box[6 * i + k] = b.nbox[i].lo[k];
            out.node_box[6 * i + 3 + k] = b.nbox[i].hi[k];
        }
    out.ref_prim.resize(b.leaf_refs.size());
    out.ref_box.resize(6 * b.leaf_refs.size());
    for (size_t r = 0; r < b.leaf_refs.size(); ++r)
    {
        out.ref_prim[r] = b.leaf_refs[r].prim;
        for (int k = 0; k < 3; ++k)
        {
            out.ref_box[6 * r + k] = b.leaf_refs[r].box.lo[k];
            out.ref_box[6 * r + 3 + k] = b.leaf_refs[r].box.hi[k];
        }
    }
    out.root = root_node;
}

}  // namespace mcrt
