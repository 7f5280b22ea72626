// Flattens a binary BVH (the library's own or the reference SplitBVH tree given
// through mcrt_bvh_tree) into the two device layouts of layout.h, depth-first.
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "host.h"

namespace mcrt {
namespace {

inline float4 f4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline float  ibits(int32_t i)
{
    float f;
    static_assert(sizeof(f) == sizeof(i), "int/float size");
    std::memcpy(&f, &i, sizeof(f));
    return f;
}

struct Flattener
{
    const BinaryTree& t;
    const float*      v;
    int64_t           num_tris;
    FlatBVH&          out;
    std::string       err;
    std::vector<int>  ref_index;  // binary node -> RefNode index

    Flattener(const BinaryTree& tree, const float* verts, int64_t n, FlatBVH& o)
        : t(tree), v(verts), num_tris(n), out(o)
    {
    }

    const int32_t* info(int node) const { return &t.node_info[6 * static_cast<size_t>(node)]; }
    const float*   box(int node) const { return &t.node_box[6 * static_cast<size_t>(node)]; }

    // reference layout: every node in DFS order with its own box
    int emit_ref(int node, int depth)
    {
        if (depth > out.max_depth) out.max_depth = depth;
        if (depth > 4096)
        {
            err = "BVH deeper than 4096 levels";
            return -1;
        }
        int idx = static_cast<int>(out.ref_nodes.size());
        out.ref_nodes.push_back(RefNode());
        const int32_t* in = info(node);
        const float*   b = box(node);
        RefNode        rn;
        if (in[0])
        {
            rn.lo = f4(b[0], b[1], b[2], ibits(~in[4]));
            rn.hi = f4(b[3], b[4], b[5], ibits(in[5]));
        }
        else
        {
            int l = emit_ref(in[1], depth + 1);
            int r = emit_ref(in[2], depth + 1);
            if (l < 0 || r < 0) return -1;
            rn.lo = f4(b[0], b[1], b[2], ibits(l));
            rn.hi = f4(b[3], b[4], b[5], ibits((r << 2) | (in[3] & 3)));
        }
        out.ref_nodes[idx] = rn;
        return idx;
    }

    // appends a leaf's triangles to fast_tris; returns the encoded child
    void emit_leaf(int node, int32_t& child, int32_t& count)
    {
        const int32_t* in = info(node);
        int            first = static_cast<int>(out.fast_tris.size() / 3);
        for (int k = 0; k < in[5]; ++k)
        {
            int32_t      p = t.ref_prim[in[4] + k];
            const float* tv = v + 9 * static_cast<int64_t>(p);
            out.fast_tris.push_back(f4(tv[0], tv[1], tv[2], ibits(p)));
            out.fast_tris.push_back(f4(tv[3], tv[4], tv[5], 0.f));
            out.fast_tris.push_back(f4(tv[6], tv[7], tv[8], 0.f));
        }
        // leaf code: ~((first << 4) | count), count <= 15
        child = ~((first << 4) | in[5]);
        count = in[5];
    }

    int emit_fast(int node)
    {
        int idx = static_cast<int>(out.fast_nodes.size());
        out.fast_nodes.push_back(FastNode());
        const int32_t* in = info(node);
        int            ch[2] = {in[1], in[2]};
        int32_t        enc[2], cnt[2] = {0, 0};
        float          lo[2][3], hi[2][3];
        for (int c = 0; c < 2; ++c)
        {
            const float* b = box(ch[c]);
            for (int k = 0; k < 3; ++k)
            {
                lo[c][k] = b[k];
                hi[c][k] = b[3 + k];
            }
            if (info(ch[c])[0])
                emit_leaf(ch[c], enc[c], cnt[c]);
            else
                enc[c] = emit_fast(ch[c]);
        }
        FastNode& fn = out.fast_nodes[idx];
        fn.n0 = f4(lo[0][0], hi[0][0], lo[0][1], hi[0][1]);
        fn.n1 = f4(lo[1][0], hi[1][0], lo[1][1], hi[1][1]);
        fn.n2 = f4(lo[0][2], hi[0][2], lo[1][2], hi[1][2]);
        fn.n3 = int4{enc[0], enc[1], cnt[0], cnt[1]};
        return idx;
    }

    bool validate()
    {
        size_t nn = t.node_info.size() / 6;
        if (t.node_box.size() != 6 * nn || t.ref_box.size() != 6 * t.ref_prim.size() || nn == 0)
        {
            err = "malformed BVH arrays";
            return false;
        }
        if (t.root < 0 || static_cast<size_t>(t.root) >= nn)
        {
            err = "BVH root out of range";
            return false;
        }
        for (size_t i = 0; i < nn; ++i)
        {
            const int32_t* in = info(static_cast<int>(i));
            if (in[0])
            {
                if (in[5] > 15)
                {
                    err = "BVH leaf with more than 15 references";
                    return false;
                }
                if (in[4] < 0 || in[5] < 0 || static_cast<size_t>(in[4]) + in[5] > t.ref_prim.size())
                {
                    err = "BVH leaf reference range out of bounds";
                    return false;
                }
            }
            else if (in[1] < 0 || in[2] < 0 || static_cast<size_t>(in[1]) >= nn || static_cast<size_t>(in[2]) >= nn ||
                     in[3] < 0 || in[3] > 2)
            {
                err = "BVH inner node child/axis out of range";
                return false;
            }
        }
        for (int32_t p : t.ref_prim)
            if (p < 0 || p >= num_tris)
            {
                err = "BVH reference primitive id out of range";
                return false;
            }
        return true;
    }

    bool run()
    {
        if (!validate()) return false;
        out.ref_nodes.reserve(t.node_info.size() / 6);
        if (emit_ref(t.root, 0) < 0) return false;
        for (size_t k = 0; k < t.ref_prim.size(); ++k)
        {
            const float* b = &t.ref_box[6 * k];
            RefPrim      rp;
            rp.lo = f4(b[0], b[1], b[2], ibits(t.ref_prim[k]));
            rp.hi = f4(b[3], b[4], b[5], 0.f);
            out.ref_prims.push_back(rp);
        }
        if (info(t.root)[0])
        {
            // a root leaf becomes a node with one leaf child and one empty child
            FastNode fn;
            int32_t  enc, cnt;
            emit_leaf(t.root, enc, cnt);
            const float* b = box(t.root);
            const float  inf = std::numeric_limits<float>::infinity();
            fn.n0 = f4(b[0], b[3], b[1], b[4]);
            fn.n1 = f4(inf, -inf, inf, -inf);
            fn.n2 = f4(b[2], b[5], inf, -inf);
            fn.n3 = int4{enc, ~0, cnt, 0};  // ~0: empty leaf (count 0)
            out.fast_nodes.push_back(fn);
        }
        else
        {
            emit_fast(t.root);
        }
        return true;
    }
};

}  // namespace

std::string flatten_tree(const BinaryTree& tree, const float* vertices, int64_t num_tris, FlatBVH& out)
{
    Flattener f(tree, vertices, num_tris, out);
    if (!f.run()) return f.err.empty() ? std::string("flatten failed") : f.err;
    return std::string();
}

}  // namespace mcrt
