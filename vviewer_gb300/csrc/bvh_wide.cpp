// Collapse of a binary BVH into compressed 8-wide nodes, the node format of
// Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs
// Through Compressed Wide BVHs" (HPG 2017): child boxes quantised to 8 bits
// per plane against a node origin and per-axis power-of-two scales, internal
// children stored contiguously, the triangles of the leaf children stored
// contiguously, and child slots assigned per ray-direction octant so that a
// ray meets the children roughly front to back when it takes them in slot
// order XOR its octant.
//
// The quantisation is exact by construction: the origin is a multiple of the
// scale and every plane origin + q * scale is representable, so the device
// reconstructs each plane without rounding and the slab test keeps the
// conservative bound of the binary nodes; every quantised box contains the
// child box it stands for.
#include "bvh_build.h"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace vvpt {
namespace {

constexpr int kWideLeafMax = 4; // triangles per leaf slot (8 slots x 4 = the 32-bit triangle mask)

// Binary subtrees of at most kWideLeafMax triangles collapse into one leaf
// slot (fuller nodes, more triangle tests per ray) when set.
#ifndef VVPT_WIDE_FLATTEN
#define VVPT_WIDE_FLATTEN 0
#endif

struct WBox {
    double lo[3] = {INFINITY, INFINITY, INFINITY};
    double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const WBox &b)
    {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    bool valid() const { return lo[0] <= hi[0]; }
    double area() const
    {
        if (!valid())
            return 0.0;
        const double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

// A child during collapse: a binary internal node, or a range of the binary
// leaf order (a leaf, or part of a leaf larger than a wide leaf slot holds).
struct CRef {
    WBox box;
    int node = -1; // binary internal node, or -1 for a primitive range
    int first = 0, count = 0;
    bool expandable() const { return node >= 0 || count > kWideLeafMax; }
};

class Collapser
{
public:
    Collapser(const BVHBuildResult &bin, const std::vector<Box3> &boxes) : m_bin(bin), m_boxes(boxes) {}

    WideBuildResult run()
    {
        // primitive range of every binary subtree (subtrees cover contiguous
        // ranges of the leaf order)
        m_first.assign(m_bin.nodes.size(), 0);
        m_count.assign(m_bin.nodes.size(), 0);
        if (!m_bin.nodes.empty())
            subtree_range(0);
        WideBuildResult out;
        m_out = &out;
        out.nodes.resize(1);
        CRef root;
        root.node = 0;
        root.box = node_box(0);
        fill(0, root, 1);
        return out;
    }

private:
    void subtree_range(int n)
    {
        const BVHNode &b = m_bin.nodes[n];
        const int idx[2] = {b.c.x, b.c.y}, cnt[2] = {b.c.z, b.c.w};
        int lo = INT32_MAX, total = 0;
        for (int k = 0; k < 2; k++) {
            if (idx[k] < 0)
                continue;
            if (cnt[k] == 0) {
                subtree_range(idx[k]);
                lo = std::min(lo, m_first[idx[k]]);
                total += m_count[idx[k]];
            } else {
                lo = std::min(lo, idx[k]);
                total += cnt[k];
            }
        }
        m_first[n] = total ? lo : 0;
        m_count[n] = total;
    }

    WBox range_box(int first, int count) const
    {
        WBox b;
        for (int k = first; k < first + count; k++) {
            const Box3 &p = m_boxes[m_bin.order[k]];
            for (int a = 0; a < 3; a++) {
                b.lo[a] = std::min(b.lo[a], (double)p.lo[a]);
                b.hi[a] = std::max(b.hi[a], (double)p.hi[a]);
            }
        }
        return b;
    }

    // the two child links of binary node `n` (empty children skipped)
    void children_of(int n, std::vector<CRef> &out) const
    {
        const BVHNode &b = m_bin.nodes[n];
        const float lo[2][3] = {{b.lxy.x, b.lxy.z, b.lrz.x}, {b.rxy.x, b.rxy.z, b.lrz.z}};
        const float hi[2][3] = {{b.lxy.y, b.lxy.w, b.lrz.y}, {b.rxy.y, b.rxy.w, b.lrz.w}};
        const int idx[2] = {b.c.x, b.c.y}, cnt[2] = {b.c.z, b.c.w};
        for (int k = 0; k < 2; k++) {
            if (idx[k] < 0)
                continue;
            CRef c;
            for (int a = 0; a < 3; a++) {
                c.box.lo[a] = lo[k][a];
                c.box.hi[a] = hi[k][a];
            }
            if (cnt[k] == 0 && (!VVPT_WIDE_FLATTEN || m_count[idx[k]] > kWideLeafMax)) {
                c.node = idx[k];
            } else if (cnt[k] == 0) {
                // a subtree of at most kWideLeafMax triangles becomes one leaf
                c.first = m_first[idx[k]];
                c.count = m_count[idx[k]];
            } else {
                c.first = idx[k];
                c.count = cnt[k];
            }
            out.push_back(c);
        }
    }

    WBox node_box(int n) const
    {
        std::vector<CRef> ch;
        children_of(n, ch);
        WBox b;
        for (const CRef &c : ch)
            b.grow(c.box);
        return b;
    }

    void expand(const CRef &r, std::vector<CRef> &out) const
    {
        if (r.node >= 0) {
            children_of(r.node, out);
            return;
        }
        const int h = r.count / 2;
        CRef a, b;
        a.first = r.first;
        a.count = h;
        a.box = range_box(a.first, a.count);
        b.first = r.first + h;
        b.count = r.count - h;
        b.box = range_box(b.first, b.count);
        out.push_back(a);
        out.push_back(b);
    }

    // Fills wide node `w` for `r` (an expandable child); its internal
    // children get consecutive wide nodes, filled afterwards (depth first).
    void fill(int w, const CRef &r, int depth)
    {
        m_out->depth = std::max(m_out->depth, depth);
        std::vector<CRef> ch;
        expand(r, ch);
        if (ch.empty()) {
            m_out->nodes[w] = WideNode{}; // an empty mesh: no child slot is valid
            return;
        }
        // greedy: open the largest expandable child while slots remain
        while (ch.size() < 8) {
            int best = -1;
            double best_area = -1.0;
            for (int k = 0; k < (int)ch.size(); k++)
                if (ch[k].expandable() && ch[k].box.area() > best_area) {
                    best = k;
                    best_area = ch[k].box.area();
                }
            if (best < 0)
                break;
            std::vector<CRef> sub;
            expand(ch[best], sub);
            if (ch.size() - 1 + sub.size() > 8)
                break;
            ch.erase(ch.begin() + best);
            ch.insert(ch.end(), sub.begin(), sub.end());
        }
        // slots: greedy assignment of (child, octant) pairs by how far the
        // child lies against the octant's diagonal
        WBox u;
        for (const CRef &c : ch)
            u.grow(c.box);
        double pc[3];
        for (int a = 0; a < 3; a++)
            pc[a] = 0.5 * (u.lo[a] + u.hi[a]);
        int slot_of[8], child_in[8];
        std::fill(slot_of, slot_of + 8, -1);
        std::fill(child_in, child_in + 8, -1);
        for (size_t done = 0; done < ch.size(); done++) {
            double best = INFINITY;
            int bc = -1, bs = -1;
            for (int c = 0; c < (int)ch.size(); c++) {
                if (slot_of[c] >= 0)
                    continue;
                for (int s = 0; s < 8; s++) {
                    if (child_in[s] >= 0)
                        continue;
                    double cost = 0.0;
                    for (int a = 0; a < 3; a++) {
                        const double d = 0.5 * (ch[c].box.lo[a] + ch[c].box.hi[a]) - pc[a];
                        cost += (s >> a & 1) ? -d : d;
                    }
                    if (cost < best) {
                        best = cost;
                        bc = c;
                        bs = s;
                    }
                }
            }
            slot_of[bc] = bs;
            child_in[bs] = bc;
        }

        WideNode n{};
        // quantisation frame per axis: origin p = k * 2^e, all planes
        // p + q * 2^e (0 <= q <= 255) exactly representable in float
        double p[3], scale[3];
        int e[3];
        for (int a = 0; a < 3; a++) {
            const double lo = u.lo[a], hi = u.hi[a];
            const double mag = std::max(std::fabs(lo), std::fabs(hi));
            int ea = -126;
            if (mag > 0.0)
                ea = std::max(ea, (int)std::ceil(std::log2(mag / (16777216.0 - 512.0))));
            if (hi > lo)
                ea = std::max(ea, (int)std::ceil(std::log2((hi - lo) / 255.0)));
            for (;;) {
                const double s = std::ldexp(1.0, ea);
                const double pa = std::floor(lo / s) * s;
                if ((hi - pa) / s <= 255.0) {
                    p[a] = pa;
                    scale[a] = s;
                    break;
                }
                ea++;
            }
            e[a] = ea;
        }
        n.px = (float)p[0];
        n.py = (float)p[1];
        n.pz = (float)p[2];
        n.ex = (uint8_t)(e[0] + 127);
        n.ey = (uint8_t)(e[1] + 127);
        n.ez = (uint8_t)(e[2] + 127);
        uint8_t *qlo[3] = {n.qlox, n.qloy, n.qloz}, *qhi[3] = {n.qhix, n.qhiy, n.qhiz};

        // internal children: consecutive wide nodes in slot order; leaf
        // children: their triangles appended in slot order
        const int child_base = (int)m_out->nodes.size();
        const uint32_t tri_base = (uint32_t)m_out->order.size();
        int n_internal = 0, tri_off = 0;
        std::vector<std::pair<int, int>> pending; // (wide node, child)
        for (int s = 0; s < 8; s++) {
            const int c = child_in[s];
            if (c < 0)
                continue;
            const CRef &cr = ch[c];
            for (int a = 0; a < 3; a++) {
                const double ql = std::floor((cr.box.lo[a] - p[a]) / scale[a]);
                const double qh = std::ceil((cr.box.hi[a] - p[a]) / scale[a]);
                qlo[a][s] = (uint8_t)std::min(255.0, std::max(0.0, ql));
                qhi[a][s] = (uint8_t)std::min(255.0, std::max(0.0, qh));
            }
            if (cr.expandable()) {
                n.imask |= (uint8_t)(1u << s);
                pending.emplace_back(child_base + n_internal, c);
                n_internal++;
            } else {
                n.meta[s] = (uint8_t)((cr.count << 5) | tri_off);
                for (int k = 0; k < cr.count; k++)
                    m_out->order.push_back(m_bin.order[cr.first + k]);
                tri_off += cr.count;
            }
        }
        n.child_base = (uint32_t)child_base;
        n.tri_base = tri_base;
        m_out->nodes[w] = n;
        m_out->nodes.resize(m_out->nodes.size() + n_internal);
        for (const auto &pc2 : pending)
            fill(pc2.first, ch[pc2.second], depth + 1);
    }

    const BVHBuildResult &m_bin;
    const std::vector<Box3> &m_boxes;
    std::vector<int> m_first, m_count;
    WideBuildResult *m_out = nullptr;
};

}  // namespace

WideBuildResult collapse_to_wide(const BVHBuildResult &bin, const std::vector<Box3> &boxes)
{
    return Collapser(bin, boxes).run();
}

}  // namespace vvpt
