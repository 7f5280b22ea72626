// Eight-child compressed BVH for the FAST traversal (WideNode, layout.h), collapsed from
// the binary tree the flattener validated.  The layout and the collapse follow Ylitie,
// Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
// BVHs" (HPG 2017); the encoding details are this library's own:
//
//  * collapse: dynamic programming over the binary tree.  cost(n, k) is the smallest SAH
//    cost of representing the subtree of n with at most k children of a wide node: n as
//    one leaf child (<= 4 triangles), n as one inner child (a wide node whose <= 8
//    children are drawn from n's descendants), or the k slots split between n's two
//    children.  A wide-node visit costs 1 and a triangle test c_tri, both weighted by
//    the surface area of the box they are reached through;
//  * slots: the children of a node are assigned to slots 0..7 so that the child in slot
//    s lies furthest back along the direction of octant s (sign bits of the direction),
//    greedily by the smallest cost dot(centre - node centre, octant direction); a ray of
//    octant o visits slots in the order slot ^ o;
//  * quantisation: per axis a power-of-two cell 2^e with 253 cells covering the node box,
//    the grid origin one cell below the box, every child plane rounded outwards and then
//    moved out by one more cell.  The device turns a quantised plane q into a ray
//    distance with one byte permute and one FMA, t = (2^23 + q) a + (b - 2^23 a), whose
//    second term is rounded once: an error below half a cell in t, covered by the extra
//    cell.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "host.h"

namespace mcrt {
namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr int    kMaxChildren = 8;

struct Box
{
    float lo[3], hi[3];
};

Box empty_box()
{
    const float inf = std::numeric_limits<float>::infinity();
    return Box{{inf, inf, inf}, {-inf, -inf, -inf}};
}

void grow(Box& a, const Box& b)
{
    for (int k = 0; k < 3; ++k)
    {
        a.lo[k] = std::min(a.lo[k], b.lo[k]);
        a.hi[k] = std::max(a.hi[k], b.hi[k]);
    }
}

double area(const Box& b)
{
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = std::max(0.0, static_cast<double>(b.hi[k]) - b.lo[k]);
    return 2.0 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
}

inline float ibits(int32_t i)
{
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

// decision of cost(n, k)
enum Kind : int8_t
{
    K_NONE = 0,     // empty subtree
    K_LEAF = 1,     // leaf child(ren) with the subtree's triangles
    K_INNER = 2,    // one inner child: n becomes a wide node
    K_SPLIT = 3,    // the k slots split between n's children (split_left of them to the left)
    K_FEWER = 4,    // same as cost(n, k - 1)
};

struct Child
{
    Box  box;
    bool inner;
    int  node;               // inner: the binary node that becomes a wide node
    std::vector<int32_t> refs;  // leaf: the references (indices into ref_prim)
};

struct Collapser
{
    const BinaryTree& t;
    const float*      v;
    FlatBVH&          out;
    double            c_tri;
    size_t            nn;
    std::vector<double>  sa;
    std::vector<int32_t> nrefs;
    std::vector<double>  cost;    // [n * 9 + k], k = 1..8
    std::vector<int8_t>  kind;    // [n * 9 + k]
    std::vector<int8_t>  left_k;  // [n * 9 + k] for K_SPLIT
    std::vector<double>  inner_cost;
    std::string          err;

    Collapser(const BinaryTree& tree, const float* verts, FlatBVH& o, double ct)
        : t(tree), v(verts), out(o), c_tri(ct), nn(tree.node_info.size() / 6)
    {
    }

    const int32_t* info(int n) const { return &t.node_info[6 * static_cast<size_t>(n)]; }
    Box            box(int n) const
    {
        const float* b = &t.node_box[6 * static_cast<size_t>(n)];
        return Box{{b[0], b[1], b[2]}, {b[3], b[4], b[5]}};
    }
    double& C(int n, int k) { return cost[static_cast<size_t>(n) * 9 + k]; }
    int8_t& K(int n, int k) { return kind[static_cast<size_t>(n) * 9 + k]; }

    // post-order over the binary tree (iterative: external trees may be deep)
    std::vector<int> post_order() const
    {
        std::vector<int> order, stack{t.root};
        order.reserve(nn);
        while (!stack.empty())
        {
            int n = stack.back();
            stack.pop_back();
            order.push_back(n);
            if (!info(n)[0])
            {
                stack.push_back(info(n)[1]);
                stack.push_back(info(n)[2]);
            }
        }
        std::reverse(order.begin(), order.end());
        return order;
    }

    // the cheapest split of k slots between the two children of inner node n
    double split_cost(int n, int k, int& best_left) const
    {
        const int l = info(n)[1], r = info(n)[2];
        const bool le = nrefs[l] == 0, re = nrefs[r] == 0;
        best_left = 0;
        if (le && re) return 0.0;
        auto c = [&](int x, int j) { return cost[static_cast<size_t>(x) * 9 + j]; };
        if (le)
        {
            best_left = 0;
            return c(r, k);
        }
        if (re)
        {
            best_left = k;
            return c(l, k);
        }
        double best = kInf;
        for (int kl = 1; kl < k; ++kl)
        {
            double v2 = c(l, kl) + c(r, k - kl);
            if (v2 < best)
            {
                best = v2;
                best_left = kl;
            }
        }
        return best;
    }

    void costs()
    {
        sa.assign(nn, 0.0);
        nrefs.assign(nn, 0);
        cost.assign(nn * 9, kInf);
        kind.assign(nn * 9, K_NONE);
        left_k.assign(nn * 9, 0);
        inner_cost.assign(nn, kInf);
        for (int n : post_order())
        {
            const int32_t* in = info(n);
            sa[n] = area(box(n));
            if (in[0])
            {
                const int r = in[5];
                nrefs[n] = r;
                if (r == 0)
                {
                    for (int k = 1; k <= kMaxChildren; ++k)
                    {
                        C(n, k) = 0.0;
                        K(n, k) = K_NONE;
                    }
                    continue;
                }
                const int    slots = (r + kWideMaxLeafTris - 1) / kWideMaxLeafTris;
                const double leaf = sa[n] * c_tri * r;
                inner_cost[n] = sa[n] + leaf;  // a wide node of `slots` leaf children
                for (int k = 1; k <= kMaxChildren; ++k)
                {
                    if (k >= slots && leaf <= inner_cost[n])
                    {
                        C(n, k) = leaf;
                        K(n, k) = K_LEAF;
                    }
                    else
                    {
                        C(n, k) = inner_cost[n];
                        K(n, k) = K_INNER;
                    }
                }
                continue;
            }
            const int l = in[1], r = in[2];
            nrefs[n] = nrefs[l] + nrefs[r];
            if (nrefs[n] == 0)
            {
                for (int k = 1; k <= kMaxChildren; ++k) C(n, k) = 0.0;
                continue;
            }
            int       kl8 = 0;
            const double d8 = split_cost(n, kMaxChildren, kl8);
            inner_cost[n] = sa[n] + d8;
            const double leaf = nrefs[n] <= kWideMaxLeafTris ? sa[n] * c_tri * nrefs[n] : kInf;
            if (leaf <= inner_cost[n])
            {
                C(n, 1) = leaf;
                K(n, 1) = K_LEAF;
            }
            else
            {
                C(n, 1) = inner_cost[n];
                K(n, 1) = K_INNER;
            }
            for (int k = 2; k <= kMaxChildren; ++k)
            {
                int          kl = 0;
                const double d = split_cost(n, k, kl);
                if (d < C(n, k - 1))
                {
                    C(n, k) = d;
                    K(n, k) = K_SPLIT;
                    left_k[static_cast<size_t>(n) * 9 + k] = static_cast<int8_t>(kl);
                }
                else
                {
                    C(n, k) = C(n, k - 1);
                    K(n, k) = K_FEWER;
                }
            }
        }
    }

    void gather_refs(int n, std::vector<int32_t>& refs) const
    {
        std::vector<int> stack{n};
        while (!stack.empty())
        {
            int x = stack.back();
            stack.pop_back();
            const int32_t* in = info(x);
            if (in[0])
                for (int k = 0; k < in[5]; ++k) refs.push_back(in[4] + k);
            else
            {
                stack.push_back(in[2]);
                stack.push_back(in[1]);
            }
        }
    }

    // leaf children of at most kWideMaxLeafTris references each, with the box of n
    void add_leaves(int n, std::vector<Child>& kids) const
    {
        std::vector<int32_t> refs;
        gather_refs(n, refs);
        for (size_t i = 0; i < refs.size(); i += kWideMaxLeafTris)
        {
            Child c;
            c.box = box(n);
            c.inner = false;
            c.node = -1;
            c.refs.assign(refs.begin() + i, refs.begin() + std::min(refs.size(), i + kWideMaxLeafTris));
            kids.push_back(c);
        }
    }

    // the children that k slots of subtree n contribute to a wide node
    void collect(int n, int k, std::vector<Child>& kids)
    {
        while (true)
        {
            const int8_t kd = K(n, k);
            if (kd == K_NONE) return;
            if (kd == K_FEWER)
            {
                --k;
                continue;
            }
            if (kd == K_LEAF)
            {
                add_leaves(n, kids);
                return;
            }
            if (kd == K_INNER)
            {
                Child c;
                c.box = box(n);
                c.inner = true;
                c.node = n;
                kids.push_back(c);
                return;
            }
            // K_SPLIT
            const int kl = left_k[static_cast<size_t>(n) * 9 + k];
            const int l = info(n)[1], r = info(n)[2];
            if (kl > 0) collect(l, kl, kids);
            if (k - kl > 0) collect(r, k - kl, kids);
            return;
        }
    }

    // the children of the wide node made from binary node n
    std::vector<Child> children_of(int n)
    {
        std::vector<Child> kids;
        const int32_t*     in = info(n);
        if (in[0])
            add_leaves(n, kids);
        else
        {
            int kl = 0;
            split_cost(n, kMaxChildren, kl);
            const int l = in[1], r = in[2];
            if (kl > 0) collect(l, kl, kids);
            if (kMaxChildren - kl > 0) collect(r, kMaxChildren - kl, kids);
        }
        return kids;
    }

    // greedy octant assignment: slot s gets the child furthest back along octant s
    static void assign_slots(const std::vector<Child>& kids, int slot_of[kMaxChildren])
    {
        const int n = static_cast<int>(kids.size());
        double    pc[3] = {0, 0, 0};
        Box       all = empty_box();
        for (const Child& c : kids) grow(all, c.box);
        for (int k = 0; k < 3; ++k) pc[k] = 0.5 * (static_cast<double>(all.lo[k]) + all.hi[k]);
        double cost[kMaxChildren][kMaxChildren];
        for (int i = 0; i < n; ++i)
            for (int s = 0; s < kMaxChildren; ++s)
            {
                double d = 0.0;
                for (int k = 0; k < 3; ++k)
                {
                    const double ck = 0.5 * (static_cast<double>(kids[i].box.lo[k]) + kids[i].box.hi[k]) - pc[k];
                    d += ((s >> k) & 1) ? -ck : ck;
                }
                cost[i][s] = d;
            }
        bool used_child[kMaxChildren] = {}, used_slot[kMaxChildren] = {};
        for (int i = 0; i < n; ++i) slot_of[i] = -1;
        for (int round = 0; round < n; ++round)
        {
            double best = kInf;
            int    bi = -1, bs = -1;
            for (int i = 0; i < n; ++i)
                if (!used_child[i])
                    for (int s = 0; s < kMaxChildren; ++s)
                        if (!used_slot[s] && cost[i][s] < best)
                        {
                            best = cost[i][s];
                            bi = i;
                            bs = s;
                        }
            if (bi < 0)  // NaN costs (degenerate boxes): first free slot
            {
                for (int i = 0; i < n && bi < 0; ++i)
                    if (!used_child[i]) bi = i;
                for (int s = 0; s < kMaxChildren && bs < 0; ++s)
                    if (!used_slot[s]) bs = s;
            }
            used_child[bi] = used_slot[bs] = true;
            slot_of[bi] = bs;
        }
    }

    // quantisation of one axis: grid origin (a float one cell below the box) and the
    // exponent of the cell, the smallest for which the box's planes, rounded outwards and
    // moved out by one more cell, stay within 0..255 of the float origin
    static void quantise_axis(float lo, float hi, float& origin, int& ebias)
    {
        double ext = static_cast<double>(hi) - lo;
        if (!(ext > 0.0)) ext = std::max(std::fabs(static_cast<double>(lo)), 1.0) * 1e-6;
        int e = static_cast<int>(std::ceil(std::log2(ext / 253.0)));
        while (std::ldexp(253.0, e) < ext) ++e;
        for (;; ++e)
        {
            const int    ec = std::max(-126, std::min(127, e));
            const double cell = std::ldexp(1.0, ec);
            const double o = static_cast<double>(lo) - cell;
            float        of = static_cast<float>(o);
            if (static_cast<double>(of) > o) of = std::nextafter(of, -std::numeric_limits<float>::infinity());
            const double qh = std::ceil((static_cast<double>(hi) - of) / cell) + 1.0;
            const double ql = std::floor((static_cast<double>(lo) - of) / cell) - 1.0;
            if ((qh <= 255.0 && ql >= 0.0) || ec == 127)
            {
                origin = of;
                ebias = ec + 127;
                return;
            }
        }
    }

    static uint8_t q_lo(float x, float origin, int ebias)
    {
        const double cell = std::ldexp(1.0, ebias - 127);
        double       q = std::floor((static_cast<double>(x) - origin) / cell) - 1.0;
        return static_cast<uint8_t>(std::max(0.0, std::min(255.0, q)));
    }
    static uint8_t q_hi(float x, float origin, int ebias)
    {
        const double cell = std::ldexp(1.0, ebias - 127);
        double       q = std::ceil((static_cast<double>(x) - origin) / cell) + 1.0;
        return static_cast<uint8_t>(std::max(0.0, std::min(255.0, q)));
    }

    bool emit()
    {
        out.wide_nodes.clear();
        out.wide_tris.clear();
        out.wide_nodes.push_back(WideNode());
        struct Work
        {
            int binary, wide, depth;
        };
        std::vector<Work> work{{t.root, 0, 1}};
        out.wide_depth = 0;
        while (!work.empty())
        {
            Work w = work.back();
            work.pop_back();
            out.wide_depth = std::max(out.wide_depth, w.depth);
            std::vector<Child> kids = nrefs[w.binary] == 0 ? std::vector<Child>() : children_of(w.binary);
            if (kids.size() > static_cast<size_t>(kMaxChildren))
            {
                err = "wide BVH: more than eight children";
                return false;
            }
            int slot_of[kMaxChildren];
            assign_slots(kids, slot_of);
            int by_slot[kMaxChildren];
            for (int s = 0; s < kMaxChildren; ++s) by_slot[s] = -1;
            for (size_t i = 0; i < kids.size(); ++i) by_slot[slot_of[i]] = static_cast<int>(i);
            Box all = empty_box();
            for (const Child& c : kids) grow(all, c.box);
            float origin[3] = {0.f, 0.f, 0.f};
            int   eb[3] = {127, 127, 127};
            if (!kids.empty())
                for (int k = 0; k < 3; ++k) quantise_axis(all.lo[k], all.hi[k], origin[k], eb[k]);
            uint8_t qlo[3][kMaxChildren], qhi[3][kMaxChildren], meta[kMaxChildren] = {};
            uint32_t imask = 0, leafmask = 0;
            const int child_base = static_cast<int>(out.wide_nodes.size());
            const int tri_base = static_cast<int>(out.wide_tris.size() / 3);
            int       ninner = 0, ntris = 0;
            std::vector<Work> next;
            for (int s = 0; s < kMaxChildren; ++s)
            {
                const int i = by_slot[s];
                for (int k = 0; k < 3; ++k)
                {
                    qlo[k][s] = 255;
                    qhi[k][s] = 0;
                }
                if (i < 0) continue;
                const Child& c = kids[i];
                for (int k = 0; k < 3; ++k)
                {
                    qlo[k][s] = q_lo(c.box.lo[k], origin[k], eb[k]);
                    qhi[k][s] = q_hi(c.box.hi[k], origin[k], eb[k]);
                }
                if (c.inner)
                {
                    imask |= 1u << s;
                    next.push_back(Work{c.node, child_base + ninner, w.depth + 1});
                    ++ninner;
                }
                else
                {
                    const int cnt = static_cast<int>(c.refs.size());
                    if (cnt < 1 || cnt > kWideMaxLeafTris || ntris + cnt > kWideMaxNodeTris)
                    {
                        err = "wide BVH: leaf child triangle count out of range";
                        return false;
                    }
                    leafmask |= 1u << s;
                    meta[s] = static_cast<uint8_t>(0x80 | ((cnt - 1) << 5) | ntris);
                    for (int32_t ref : c.refs)
                    {
                        const int32_t p = t.ref_prim[ref];
                        const float*  tv = v + 9 * static_cast<int64_t>(p);
                        out.wide_tris.push_back(float4{tv[0], tv[1], tv[2], ibits(p)});
                        out.wide_tris.push_back(float4{tv[3], tv[4], tv[5], 0.f});
                        out.wide_tris.push_back(float4{tv[6], tv[7], tv[8], 0.f});
                    }
                    ntris += cnt;
                }
            }
            out.wide_nodes.resize(out.wide_nodes.size() + ninner);
            auto pack = [](const uint8_t* b) {
                return static_cast<int32_t>(static_cast<uint32_t>(b[0]) | static_cast<uint32_t>(b[1]) << 8 |
                                            static_cast<uint32_t>(b[2]) << 16 | static_cast<uint32_t>(b[3]) << 24);
            };
            WideNode& wn = out.wide_nodes[w.wide];
            wn.w0 = float4{origin[0], origin[1], origin[2],
                           ibits(static_cast<int32_t>(static_cast<uint32_t>(eb[0]) | static_cast<uint32_t>(eb[1]) << 8 |
                                                      static_cast<uint32_t>(eb[2]) << 16 | imask << 24))};
            wn.w1 = int4{child_base, tri_base, pack(meta), pack(meta + 4)};
            wn.w2 = int4{pack(qlo[0]), pack(qlo[0] + 4), pack(qlo[1]), pack(qlo[1] + 4)};
            wn.w3 = int4{pack(qlo[2]), pack(qlo[2] + 4), pack(qhi[0]), pack(qhi[0] + 4)};
            wn.w4 = int4{pack(qhi[1]), pack(qhi[1] + 4), pack(qhi[2]), pack(qhi[2] + 4)};
            wn.w5 = int4{static_cast<int32_t>(leafmask), 0, 0, 0};
            // depth-first: the children's blocks follow their parent's
            for (auto it = next.rbegin(); it != next.rend(); ++it) work.push_back(*it);
        }
        return true;
    }
};

}  // namespace

std::string build_wide(const BinaryTree& tree, const float* vertices, int64_t num_tris, FlatBVH& out, float c_tri)
{
    Collapser c(tree, vertices, out, c_tri);
    c.costs();
    if (!c.emit()) return c.err;
    int depth = 0;
    std::string e = validate_wide(out.wide_nodes, out.wide_tris, num_tris, &depth);
    if (!e.empty()) return e;
    out.wide_depth = depth;
    return std::string();
}

std::string validate_wide(const std::vector<WideNode>& nodes, const std::vector<float4>& tris, int64_t num_prims,
                          int* depth)
{
    const int64_t nn = static_cast<int64_t>(nodes.size());
    const int64_t nt = static_cast<int64_t>(tris.size() / 3);
    if (nn == 0 || tris.size() % 3 != 0) return "wide BVH: empty or malformed arrays";
    std::vector<int> level(static_cast<size_t>(nn), 0);
    std::vector<uint8_t> seen(static_cast<size_t>(nn), 0);
    level[0] = 1;
    seen[0] = 1;
    int deepest = 1;
    // nodes are written parents first (every child block lies after its parent)
    for (int64_t i = 0; i < nn; ++i)
    {
        if (!seen[i]) return "wide BVH: node " + std::to_string(i) + " unreachable";
        const WideNode& w = nodes[i];
        uint32_t        bits;
        std::memcpy(&bits, &w.w0.w, 4);
        const uint32_t imask = bits >> 24, leafmask = static_cast<uint32_t>(w.w5.x);
        if ((imask & leafmask) != 0 || leafmask > 0xffu) return "wide BVH: slot both inner and leaf";
        const int64_t cb = w.w1.x, tb = w.w1.y;
        const int     ninner = __builtin_popcount(imask);
        if (ninner > 0 && (cb <= i || cb + ninner > nn)) return "wide BVH: child block out of range";
        for (int k = 0; k < ninner; ++k)
        {
            if (seen[cb + k]) return "wide BVH: node with two parents";
            seen[cb + k] = 1;
            level[cb + k] = level[i] + 1;
            deepest = std::max(deepest, level[i] + 1);
        }
        const uint32_t meta[2] = {static_cast<uint32_t>(w.w1.z), static_cast<uint32_t>(w.w1.w)};
        for (int s = 0; s < 8; ++s)
        {
            const uint32_t m = (meta[s >> 2] >> (8 * (s & 3))) & 0xffu;
            const bool     leaf = (leafmask >> s) & 1u;
            if (leaf != ((m & 0x80u) != 0)) return "wide BVH: leaf mask and meta disagree";
            if (!leaf) continue;
            const int first = m & 31, cnt = ((m >> 5) & 3) + 1;
            if (first + cnt > kWideMaxNodeTris || tb < 0 || tb + first + cnt > nt)
                return "wide BVH: leaf triangles out of range";
            for (int k = 0; k < cnt; ++k)
            {
                int32_t p;
                std::memcpy(&p, &tris[3 * (tb + first + k)].w, 4);
                if (p < 0 || p >= num_prims) return "wide BVH: primitive id out of range";
            }
        }
    }
    if (depth) *depth = deepest;
    return std::string();
}

}  // namespace mcrt
