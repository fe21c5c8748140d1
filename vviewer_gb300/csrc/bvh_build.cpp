// Binned-SAH BVH build on the host. SAH costs are accumulated in FP64 (areas
// of large scenes differ by many orders of magnitude); boxes stay FP32.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <future>
#include <thread>

namespace vvpt {
namespace {

struct Bounds {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const Box3 &b)
    {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow(const Bounds &b)
    {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow_point(const float p[3])
    {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    bool valid() const { return lo[0] <= hi[0]; }
    double area() const
    {
        if (!valid())
            return 0.0;
        double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct Link {
    int index = -1; // node index or first primitive
    int count = 0;  // >0 leaf
    Bounds box;
};

class Builder
{
public:
    Builder(const std::vector<Box3> &boxes, const BVHBuildOptions &opt)
        : m_boxes(boxes), m_opt(opt)
    {
        size_t n = boxes.size();
        m_centroids.resize(n * 3);
        for (size_t i = 0; i < n; i++)
            for (int a = 0; a < 3; a++)
                m_centroids[i * 3 + a] = 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]);
    }

    // Builds the subtree over order[begin, end) into `nodes` (appending).
    // Returns the link a parent stores for this range.
    Link build(std::vector<uint32_t> &order, std::vector<BVHNode> &nodes, int begin, int end, int depth, int &max_depth)
    {
        Link link;
        Bounds box, cbox;
        for (int i = begin; i < end; i++) {
            box.grow(m_boxes[order[i]]);
            cbox.grow_point(&m_centroids[order[i] * 3]);
        }
        link.box = box;
        int n = end - begin;
        max_depth = std::max(max_depth, depth);
        if (n <= 1 || depth >= m_opt.max_depth) {
            link.index = begin;
            link.count = n;
            return link;
        }

        int axis = -1, split_bin = -1;
        double best_cost = DBL_MAX;
        const int B = m_opt.bins;
        std::vector<Bounds> bin_box(B);
        std::vector<int> bin_cnt(B);
        std::vector<double> right_area(B);
        std::vector<int> right_cnt(B);
        for (int a = 0; a < 3; a++) {
            float extent = cbox.hi[a] - cbox.lo[a];
            if (!(extent > 0.0f))
                continue;
            std::fill(bin_box.begin(), bin_box.end(), Bounds());
            std::fill(bin_cnt.begin(), bin_cnt.end(), 0);
            double scale = (double)B / extent;
            for (int i = begin; i < end; i++) {
                uint32_t p = order[i];
                int b = (int)(((double)m_centroids[p * 3 + a] - cbox.lo[a]) * scale);
                b = std::min(std::max(b, 0), B - 1);
                bin_box[b].grow(m_boxes[p]);
                bin_cnt[b]++;
            }
            Bounds acc;
            int cnt = 0;
            for (int b = B - 1; b > 0; b--) {
                acc.grow(bin_box[b]);
                cnt += bin_cnt[b];
                right_area[b] = acc.area();
                right_cnt[b] = cnt;
            }
            acc = Bounds();
            cnt = 0;
            for (int b = 0; b < B - 1; b++) {
                acc.grow(bin_box[b]);
                cnt += bin_cnt[b];
                int rc = right_cnt[b + 1];
                if (cnt == 0 || rc == 0)
                    continue;
                double cost = acc.area() * cnt + right_area[b + 1] * rc;
                if (cost < best_cost) {
                    best_cost = cost;
                    axis = a;
                    split_bin = b;
                }
            }
        }

        double parent_area = box.area();
        double split_cost = m_opt.cost_traversal +
                            (parent_area > 0.0 ? best_cost / parent_area : (double)n) * m_opt.cost_intersect;
        double leaf_cost = (double)n * m_opt.cost_intersect;
        if (axis >= 0 && n <= m_opt.max_leaf && leaf_cost <= split_cost) {
            link.index = begin;
            link.count = n;
            return link;
        }

        int mid;
        if (axis < 0) {
            // all centroids coincide: split by index
            if (n <= m_opt.max_leaf) {
                link.index = begin;
                link.count = n;
                return link;
            }
            mid = begin + n / 2;
        } else {
            double scale = (double)B / (cbox.hi[axis] - cbox.lo[axis]);
            auto it = std::partition(order.begin() + begin, order.begin() + end, [&](uint32_t p) {
                int b = (int)(((double)m_centroids[p * 3 + axis] - cbox.lo[axis]) * scale);
                b = std::min(std::max(b, 0), B - 1);
                return b <= split_bin;
            });
            mid = (int)(it - order.begin());
            if (mid == begin || mid == end)
                mid = begin + n / 2;
        }

        int node_index = (int)nodes.size();
        nodes.emplace_back();
        Link l, r;
        if (n > 65536 && m_parallel_budget.fetch_sub(1) > 0) {
            // large subtrees: build the left half on another thread into its
            // own arrays, then splice
            std::vector<BVHNode> left_nodes;
            int left_depth = 0;
            auto fut = std::async(std::launch::async, [&]() {
                return build(order, left_nodes, begin, mid, depth + 1, left_depth);
            });
            r = build(order, nodes, mid, end, depth + 1, max_depth);
            l = fut.get();
            max_depth = std::max(max_depth, left_depth);
            if (l.count == 0 && l.index >= 0) {
                int shift = (int)nodes.size();
                for (BVHNode &nd : left_nodes) {
                    if (nd.c.z == 0 && nd.c.x >= 0)
                        nd.c.x += shift;
                    if (nd.c.w == 0 && nd.c.y >= 0)
                        nd.c.y += shift;
                }
                l.index += shift;
                nodes.insert(nodes.end(), left_nodes.begin(), left_nodes.end());
            }
        } else {
            if (n > 65536)
                m_parallel_budget.fetch_add(1);
            l = build(order, nodes, begin, mid, depth + 1, max_depth);
            r = build(order, nodes, mid, end, depth + 1, max_depth);
        }
        write_node(nodes[node_index], l, r);
        link.index = node_index;
        link.count = 0;
        return link;
    }

    static void write_node(BVHNode &nd, const Link &l, const Link &r)
    {
        auto box_or_empty = [](const Link &k, float *lo, float *hi) {
            for (int a = 0; a < 3; a++) {
                lo[a] = k.box.valid() ? k.box.lo[a] : 1.0f;
                hi[a] = k.box.valid() ? k.box.hi[a] : -1.0f; // empty box never hit
            }
        };
        float llo[3], lhi[3], rlo[3], rhi[3];
        box_or_empty(l, llo, lhi);
        box_or_empty(r, rlo, rhi);
        nd.lxy = {llo[0], lhi[0], llo[1], lhi[1]};
        nd.rxy = {rlo[0], rhi[0], rlo[1], rhi[1]};
        nd.lrz = {llo[2], lhi[2], rlo[2], rhi[2]};
        nd.c = {l.index, r.index, l.count, r.count};
        if (l.count == 0 && l.index < 0)
            nd.c.x = -1;
        if (r.count == 0 && r.index < 0)
            nd.c.y = -1;
    }

    std::atomic<int> m_parallel_budget{0};

private:
    const std::vector<Box3> &m_boxes;
    const BVHBuildOptions &m_opt;
    std::vector<float> m_centroids;
};

}  // namespace

BVHBuildResult build_bvh2(const std::vector<Box3> &boxes, const BVHBuildOptions &opt)
{
    BVHBuildResult res;
    int n = (int)boxes.size();
    res.order.resize(n);
    for (int i = 0; i < n; i++)
        res.order[i] = (uint32_t)i;
    res.nodes.reserve(n > 0 ? (size_t)n : 1);

    Builder builder(boxes, opt);
    int threads = opt.threads > 0 ? opt.threads : (int)std::thread::hardware_concurrency();
    builder.m_parallel_budget.store(std::max(0, threads - 1));

    if (n == 0) {
        BVHNode root{};
        Link empty;
        Builder::write_node(root, empty, empty);
        res.nodes.push_back(root);
        return res;
    }
    int depth = 0;
    Link top = builder.build(res.order, res.nodes, 0, n, 0, depth);
    if (top.count > 0) {
        // the whole input is one leaf: wrap it in a root with an empty sibling
        BVHNode root{};
        Link empty;
        Builder::write_node(root, top, empty);
        res.nodes.insert(res.nodes.begin(), root);
    } else if (top.index != 0) {
        // root must be node 0 (it is, since the first allocated node is the root)
    }
    res.depth = depth + 1;
    return res;
}

}  // namespace vvpt
