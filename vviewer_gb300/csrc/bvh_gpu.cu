// GPU binned-SAH BVH builder: the same binary BVH (BVHNode layout, leaf order)
// as build_bvh2 in bvh_build.cpp, built top down one tree level per round of
// kernels instead of one node at a time on the host.
//
// A task is an inner node to split: a range of positions in the primitive
// order array and its primitives' centroid bounds. Per level:
//   k_bin        every primitive of every task adds its box and centroid to
//                32 bins per axis of its task (shared-memory bins when a whole
//                block of positions belongs to one task, global atomics else)
//   k_split      one thread per task: SAH over the 31 candidate planes per
//                axis (surface area x count on both sides), or the median when
//                all centroids coincide
//   k_partition  every primitive moves to its side (per-task cursors)
//   k_emit       the task's node is written (both children's boxes and links);
//                children above the leaf size become next-level tasks, smaller
//                ones are finished by the same thread (split while the SAH
//                says so, as the host builder does)
// The host only reads the task count per level. Positions inside a leaf keep
// the order the partition left them in, so the build is not deterministic
// across runs; traversal results do not depend on it (exact closest hit under
// the (t, instance, primitive) order).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "bvh_build.h"

namespace vvpt {

namespace {

constexpr int kBins = 32;

struct GBox {
    float lo[3], hi[3];
};

struct Task {
    int begin, end, node, depth;
    float cmin[3], cmax[3];
};

// per task, axis, bin: count, box lo/hi, centroid lo/hi (float bits as
// order-preserving ints for atomic min/max)
struct BinStat {
    int count;
    int blo[3], bhi[3];
    int clo[3], chi[3];
};

struct Split {
    int axis, bin;       // left = bins [0, bin], right = (bin, 31]; axis -1: median split
    int nl;              // primitives on the left
    GBox lbox, rbox;     // children's boxes
    float lcmin[3], lcmax[3], rcmin[3], rcmax[3]; // children's centroid bounds
};

__device__ __forceinline__ int f2o(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

__device__ __forceinline__ int bin_of(float c, float lo, float hi)
{
    const float ext = hi - lo;
    if (!(ext > 0.0f))
        return 0;
    const int b = (int)((c - lo) * ((float)kBins / ext));
    return min(max(b, 0), kBins - 1);
}

__global__ void k_init(const GBox *boxes, int n, int *idx, int *task_of, float4 *cent)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        idx[i] = i;
        task_of[i] = 0;
        const GBox &b = boxes[i];
        cent[i] = make_float4(0.5f * (b.lo[0] + b.hi[0]), 0.5f * (b.lo[1] + b.hi[1]), 0.5f * (b.lo[2] + b.hi[2]), 0.0f);
    }
}

__global__ void k_clear_bins(BinStat *bins, int nstats)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nstats; i += gridDim.x * blockDim.x) {
        BinStat &b = bins[i];
        b.count = 0;
        for (int a = 0; a < 3; a++) {
            b.blo[a] = b.clo[a] = f2o(FLT_MAX);
            b.bhi[a] = b.chi[a] = f2o(-FLT_MAX);
        }
    }
}

__device__ __forceinline__ void add_to_bin(BinStat &s, const GBox &b, const float4 &c, bool shared_mem)
{
    (void)shared_mem;
    atomicAdd(&s.count, 1);
    for (int a = 0; a < 3; a++) {
        atomicMin(&s.blo[a], f2o(b.lo[a]));
        atomicMax(&s.bhi[a], f2o(b.hi[a]));
    }
    atomicMin(&s.clo[0], f2o(c.x));
    atomicMax(&s.chi[0], f2o(c.x));
    atomicMin(&s.clo[1], f2o(c.y));
    atomicMax(&s.chi[1], f2o(c.y));
    atomicMin(&s.clo[2], f2o(c.z));
    atomicMax(&s.chi[2], f2o(c.z));
}

// Blocks of 256 positions; a block whose positions all belong to one task
// bins in shared memory and flushes once.
__global__ void __launch_bounds__(256) k_bin(const GBox *boxes, const float4 *cent, const int *idx, const int *task_of,
                                             int n, const Task *tasks, BinStat *bins)
{
    __shared__ BinStat sb[3 * kBins];
    __shared__ int first_task, uniform;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = p < n ? task_of[p] : -1;
    if (threadIdx.x == 0) {
        first_task = t;
        uniform = 1;
    }
    __syncthreads();
    if (t != first_task)
        uniform = 0;
    __syncthreads();
    const bool use_shared = uniform && first_task >= 0;
    if (use_shared) {
        for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
            BinStat &b = sb[i];
            b.count = 0;
            for (int a = 0; a < 3; a++) {
                b.blo[a] = b.clo[a] = f2o(FLT_MAX);
                b.bhi[a] = b.chi[a] = f2o(-FLT_MAX);
            }
        }
        __syncthreads();
    }
    if (t >= 0) {
        const Task &T = tasks[t];
        const int prim = idx[p];
        const GBox b = boxes[prim];
        const float4 c = cent[prim];
        const float cc[3] = {c.x, c.y, c.z};
        for (int a = 0; a < 3; a++) {
            const int k = a * kBins + bin_of(cc[a], T.cmin[a], T.cmax[a]);
            add_to_bin(use_shared ? sb[k] : bins[(size_t)t * 3 * kBins + k], b, c, use_shared);
        }
    }
    if (use_shared) {
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
            const BinStat &s = sb[i];
            if (s.count == 0)
                continue;
            BinStat &g = bins[(size_t)first_task * 3 * kBins + i];
            atomicAdd(&g.count, s.count);
            for (int a = 0; a < 3; a++) {
                atomicMin(&g.blo[a], s.blo[a]);
                atomicMax(&g.bhi[a], s.bhi[a]);
                atomicMin(&g.clo[a], s.clo[a]);
                atomicMax(&g.chi[a], s.chi[a]);
            }
        }
    }
}

__device__ __forceinline__ float half_area(const float lo[3], const float hi[3])
{
    const float dx = fmaxf(hi[0] - lo[0], 0.0f), dy = fmaxf(hi[1] - lo[1], 0.0f), dz = fmaxf(hi[2] - lo[2], 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_split(const Task *tasks, int ntasks, const BinStat *bins, Split *splits)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks)
        return;
    const BinStat *B = bins + (size_t)t * 3 * kBins;
    Split best;
    best.axis = -1;
    best.bin = 0;
    best.nl = (tasks[t].end - tasks[t].begin) / 2;
    double best_cost = 1e300;
    for (int a = 0; a < 3; a++) {
        if (!(tasks[t].cmax[a] > tasks[t].cmin[a]))
            continue;
        // right-to-left sweep: area x count of the right side of plane k
        double rcost[kBins];
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        int cnt = 0;
        for (int k = kBins - 1; k > 0; k--) {
            const BinStat &s = B[a * kBins + k];
            if (s.count) {
                for (int j = 0; j < 3; j++) {
                    lo[j] = fminf(lo[j], o2f(s.blo[j]));
                    hi[j] = fmaxf(hi[j], o2f(s.bhi[j]));
                }
                cnt += s.count;
            }
            rcost[k] = cnt ? (double)half_area(lo, hi) * cnt : 0.0;
        }
        float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        int lc = 0;
        for (int k = 0; k < kBins - 1; k++) {
            const BinStat &s = B[a * kBins + k];
            if (s.count) {
                for (int j = 0; j < 3; j++) {
                    llo[j] = fminf(llo[j], o2f(s.blo[j]));
                    lhi[j] = fmaxf(lhi[j], o2f(s.bhi[j]));
                }
                lc += s.count;
            }
            const int rc = tasks[t].end - tasks[t].begin - lc;
            if (lc == 0 || rc == 0)
                continue;
            const double cost = (double)half_area(llo, lhi) * lc + rcost[k + 1];
            if (cost < best_cost) {
                best_cost = cost;
                best.axis = a;
                best.bin = k;
                best.nl = lc;
            }
        }
    }
    // children's boxes and centroid bounds from the bins (median split: from
    // the task's bounds; k_emit recomputes nothing for it)
    for (int j = 0; j < 3; j++) {
        best.lbox.lo[j] = best.rbox.lo[j] = best.lcmin[j] = best.rcmin[j] = FLT_MAX;
        best.lbox.hi[j] = best.rbox.hi[j] = best.lcmax[j] = best.rcmax[j] = -FLT_MAX;
    }
    if (best.axis >= 0) {
        for (int k = 0; k < kBins; k++) {
            const BinStat &s = B[best.axis * kBins + k];
            if (!s.count)
                continue;
            GBox &bx = k <= best.bin ? best.lbox : best.rbox;
            float *cl = k <= best.bin ? best.lcmin : best.rcmin;
            float *ch = k <= best.bin ? best.lcmax : best.rcmax;
            for (int j = 0; j < 3; j++) {
                bx.lo[j] = fminf(bx.lo[j], o2f(s.blo[j]));
                bx.hi[j] = fmaxf(bx.hi[j], o2f(s.bhi[j]));
                cl[j] = fminf(cl[j], o2f(s.clo[j]));
                ch[j] = fmaxf(ch[j], o2f(s.chi[j]));
            }
        }
    }
    splits[t] = best;
}

// Median splits (all centroids equal) keep the order: the first nl
// positions go left. Otherwise each primitive moves to its side.
__global__ void k_partition(const GBox *boxes, const float4 *cent, const int *idx_in, const int *task_of_in, int n,
                            const Task *tasks, const Split *splits, int *cursors, int *idx_out, int *side_out,
                            GBox *median_boxes)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int t = task_of_in[p];
        if (t < 0) {
            idx_out[p] = idx_in[p];
            side_out[p] = -1;
            continue;
        }
        const Task &T = tasks[t];
        const Split &S = splits[t];
        const int prim = idx_in[p];
        bool left;
        if (S.axis < 0) {
            left = p - T.begin < S.nl;
        } else {
            const float4 c = cent[prim];
            const float cc = S.axis == 0 ? c.x : (S.axis == 1 ? c.y : c.z);
            left = bin_of(cc, T.cmin[S.axis], T.cmax[S.axis]) <= S.bin;
        }
        const int dst = left ? T.begin + atomicAdd(&cursors[2 * t], 1) : T.begin + S.nl + atomicAdd(&cursors[2 * t + 1], 1);
        idx_out[dst] = prim;
        side_out[dst] = 2 * t + (left ? 0 : 1);
        if (S.axis < 0) {
            // median split: children boxes accumulated here
            const GBox b = boxes[prim];
            const float4 c = cent[prim];
            GBox &m = median_boxes[2 * t + (left ? 0 : 1)];
            int *mi = reinterpret_cast<int *>(&m);
            for (int j = 0; j < 3; j++) {
                atomicMin(&mi[j], f2o(b.lo[j]));
                atomicMax(&mi[3 + j], f2o(b.hi[j]));
            }
            (void)c;
        }
    }
}

__global__ void k_clear_median(GBox *m, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int *mi = reinterpret_cast<int *>(&m[i]);
        for (int j = 0; j < 3; j++) {
            mi[j] = f2o(FLT_MAX);
            mi[3 + j] = f2o(-FLT_MAX);
        }
    }
}

// A child of at most max_leaf primitives is finished by its parent's thread
// with the same rule as the host builder: split while the SAH says a split
// is cheaper than the leaf (traversal cost 1, intersection cost 1 per
// primitive); with so few primitives the candidate planes are the gaps
// between the sorted centroids. Returns the parent's link and count.
__device__ void small_subtree(int b, int n, int depth, int *idx, const GBox *boxes, const float4 *cent,
                              BVHNode *nodes, int *counters, int &link, int &count, GBox &box)
{
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = 0; i < n; i++) {
        const GBox g = boxes[idx[b + i]];
        for (int j = 0; j < 3; j++) {
            lo[j] = fminf(lo[j], g.lo[j]);
            hi[j] = fmaxf(hi[j], g.hi[j]);
        }
    }
    for (int j = 0; j < 3; j++) {
        box.lo[j] = lo[j];
        box.hi[j] = hi[j];
    }
    link = b;
    count = n;
    if (n <= 1)
        return;
    const double parent_area = (double)half_area(lo, hi);
    double best = 1e300;
    int best_axis = -1, best_k = 0;
    int order[8];
    for (int a = 0; a < 3; a++) {
        // sort this range's positions by centroid on axis a (n <= 8)
        for (int i = 0; i < n; i++)
            order[i] = idx[b + i];
        for (int i = 1; i < n; i++) {
            const int x = order[i];
            const float4 cx = cent[x];
            const float vx = a == 0 ? cx.x : (a == 1 ? cx.y : cx.z);
            int j = i - 1;
            while (j >= 0) {
                const float4 cj = cent[order[j]];
                const float vj = a == 0 ? cj.x : (a == 1 ? cj.y : cj.z);
                if (vj <= vx)
                    break;
                order[j + 1] = order[j];
                j--;
            }
            order[j + 1] = x;
        }
        for (int k = 1; k < n; k++) {
            float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            float rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            for (int i = 0; i < n; i++) {
                const GBox g = boxes[order[i]];
                float *l = i < k ? llo : rlo, *h = i < k ? lhi : rhi;
                for (int j = 0; j < 3; j++) {
                    l[j] = fminf(l[j], g.lo[j]);
                    h[j] = fmaxf(h[j], g.hi[j]);
                }
            }
            const double cost = (double)half_area(llo, lhi) * k + (double)half_area(rlo, rhi) * (n - k);
            if (cost < best) {
                best = cost;
                best_axis = a;
                best_k = k;
            }
        }
    }
    const double split_cost = 1.0 + (parent_area > 0.0 ? best / parent_area : (double)n);
    if (best_axis < 0 || (double)n <= split_cost)
        return; // leaf
    // reorder the range by the best axis and build both sides
    for (int i = 0; i < n; i++)
        order[i] = idx[b + i];
    for (int i = 1; i < n; i++) {
        const int x = order[i];
        const float4 cx = cent[x];
        const float vx = best_axis == 0 ? cx.x : (best_axis == 1 ? cx.y : cx.z);
        int j = i - 1;
        while (j >= 0) {
            const float4 cj = cent[order[j]];
            const float vj = best_axis == 0 ? cj.x : (best_axis == 1 ? cj.y : cj.z);
            if (vj <= vx)
                break;
            order[j + 1] = order[j];
            j--;
        }
        order[j + 1] = x;
    }
    for (int i = 0; i < n; i++)
        idx[b + i] = order[i];
    const int node = atomicAdd(&counters[0], 1);
    int ll, lc, rl, rc;
    GBox lb, rb;
    small_subtree(b, best_k, depth + 1, idx, boxes, cent, nodes, counters, ll, lc, lb);
    small_subtree(b + best_k, n - best_k, depth + 1, idx, boxes, cent, nodes, counters, rl, rc, rb);
    atomicMax(&counters[2], depth + 1);
    BVHNode nd;
    nd.lxy = make_float4(lb.lo[0], lb.hi[0], lb.lo[1], lb.hi[1]);
    nd.rxy = make_float4(rb.lo[0], rb.hi[0], rb.lo[1], rb.hi[1]);
    nd.lrz = make_float4(lb.lo[2], lb.hi[2], rb.lo[2], rb.hi[2]);
    nd.c = make_int4(ll, rl, lc, rc);
    nodes[node] = nd;
    link = node;
    count = 0;
}

// One thread per task: the node record, child tasks for children above the
// leaf size (small children finished here); child task ids go to
// child_task[2t + side].
__global__ void k_emit(const Task *tasks, int ntasks, Split *splits, const GBox *median_boxes, BVHNode *nodes,
                       int *counters /* [0] nodes, [1] next tasks, [2] max depth */, Task *next, int *child_task,
                       int max_leaf, int max_depth, int *idx, const GBox *boxes, const float4 *cent)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks)
        return;
    const Task &T = tasks[t];
    Split &S = splits[t];
    if (S.axis < 0) {
        // median: boxes from the partition's atomics; centroid bounds equal
        for (int side = 0; side < 2; side++) {
            const int *mi = reinterpret_cast<const int *>(&median_boxes[2 * t + side]);
            GBox &bx = side == 0 ? S.lbox : S.rbox;
            for (int j = 0; j < 3; j++) {
                bx.lo[j] = o2f(mi[j]);
                bx.hi[j] = o2f(mi[3 + j]);
            }
        }
        for (int j = 0; j < 3; j++) {
            S.lcmin[j] = S.rcmin[j] = T.cmin[j];
            S.lcmax[j] = S.rcmax[j] = T.cmax[j];
        }
    }
    int link[2], cnt[2];
    for (int side = 0; side < 2; side++) {
        const int b = side == 0 ? T.begin : T.begin + S.nl;
        const int e = side == 0 ? T.begin + S.nl : T.end;
        const int n = e - b;
        child_task[2 * t + side] = -1;
        if (T.depth + 1 >= max_depth) {
            link[side] = b;
            cnt[side] = n;
        } else if (n <= max_leaf && n <= 8) {
            GBox bx;
            small_subtree(b, n, T.depth + 1, idx, boxes, cent, nodes, counters, link[side], cnt[side], bx);
        } else {
            const int node = atomicAdd(&counters[0], 1);
            const int nt = atomicAdd(&counters[1], 1);
            Task c;
            c.begin = b;
            c.end = e;
            c.node = node;
            c.depth = T.depth + 1;
            for (int j = 0; j < 3; j++) {
                c.cmin[j] = side == 0 ? S.lcmin[j] : S.rcmin[j];
                c.cmax[j] = side == 0 ? S.lcmax[j] : S.rcmax[j];
            }
            next[nt] = c;
            link[side] = node;
            cnt[side] = 0;
            child_task[2 * t + side] = nt;
        }
    }
    atomicMax(&counters[2], T.depth + 1);
    BVHNode nd;
    nd.lxy = make_float4(S.lbox.lo[0], S.lbox.hi[0], S.lbox.lo[1], S.lbox.hi[1]);
    nd.rxy = make_float4(S.rbox.lo[0], S.rbox.hi[0], S.rbox.lo[1], S.rbox.hi[1]);
    nd.lrz = make_float4(S.lbox.lo[2], S.lbox.hi[2], S.rbox.lo[2], S.rbox.hi[2]);
    nd.c = make_int4(link[0], link[1], cnt[0], cnt[1]);
    nodes[T.node] = nd;
}

// positions of child tasks get their new task id; leaf positions -1
__global__ void k_retask(const int *side_in, const int *child_task, int n, int *task_of_out)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int s = side_in[p];
        task_of_out[p] = s < 0 ? -1 : child_task[s];
    }
}

struct DevMem {
    void *p = nullptr;
    ~DevMem()
    {
        if (p)
            cudaFree(p);
    }
    template <class T>
    T *as() const
    {
        return reinterpret_cast<T *>(p);
    }
};

int grid_of(long n) { return (int)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 32)); }

}  // namespace

bool build_bvh2_gpu(const std::vector<Box3> &boxes, const BVHBuildOptions &opt, cudaStream_t s, BVHBuildResult &out,
                    std::string &err)
{
    const int n = (int)boxes.size();
    if (n <= opt.max_leaf)
        return false; // the host builder handles trivial trees
    auto ck = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = std::string("GPU BVH build: ") + what + ": " + cudaGetErrorString(e);
            return false;
        }
        return true;
    };
    const int max_nodes = std::max(1, n); // a binary tree whose leaves hold >= 1 primitive has < n inner nodes
    DevMem d_boxes, d_cent, d_idx[2], d_task_of[2], d_side, d_tasks[2], d_bins, d_splits, d_cursors, d_nodes,
        d_counters, d_child, d_median;
    if (!ck(cudaMalloc(&d_boxes.p, sizeof(GBox) * n), "alloc") || !ck(cudaMalloc(&d_cent.p, sizeof(float4) * n), "alloc") ||
        !ck(cudaMalloc(&d_idx[0].p, 4ull * n), "alloc") || !ck(cudaMalloc(&d_idx[1].p, 4ull * n), "alloc") ||
        !ck(cudaMalloc(&d_task_of[0].p, 4ull * n), "alloc") || !ck(cudaMalloc(&d_task_of[1].p, 4ull * n), "alloc") ||
        !ck(cudaMalloc(&d_side.p, 4ull * n), "alloc") || !ck(cudaMalloc(&d_nodes.p, sizeof(BVHNode) * max_nodes), "alloc") ||
        !ck(cudaMalloc(&d_counters.p, 16), "alloc"))
        return false;
    static_assert(sizeof(GBox) == sizeof(Box3), "box layout");
    if (!ck(cudaMemcpyAsync(d_boxes.p, boxes.data(), sizeof(GBox) * n, cudaMemcpyHostToDevice, s), "upload"))
        return false;
    k_init<<<grid_of(n), 256, 0, s>>>(d_boxes.as<GBox>(), n, d_idx[0].as<int>(), d_task_of[0].as<int>(),
                                      d_cent.as<float4>());
    // root task: centroid bounds on the host (one pass over the boxes)
    Task root{};
    root.begin = 0;
    root.end = n;
    root.node = 0;
    root.depth = 0;
    for (int j = 0; j < 3; j++) {
        root.cmin[j] = FLT_MAX;
        root.cmax[j] = -FLT_MAX;
    }
    for (const Box3 &b : boxes)
        for (int j = 0; j < 3; j++) {
            const float c = 0.5f * (b.lo[j] + b.hi[j]);
            root.cmin[j] = std::min(root.cmin[j], c);
            root.cmax[j] = std::max(root.cmax[j], c);
        }
    int ntasks = 1, cap = 1;
    auto ensure_tasks = [&](int need) {
        if (need <= cap && d_tasks[0].p)
            return true;
        cap = std::max(need, cap * 2);
        for (auto *m : {&d_tasks[0], &d_tasks[1]}) {
            if (m->p)
                cudaFree(m->p);
            m->p = nullptr;
        }
        for (auto *m : {&d_bins, &d_splits, &d_cursors, &d_child, &d_median}) {
            if (m->p)
                cudaFree(m->p);
            m->p = nullptr;
        }
        return ck(cudaMalloc(&d_tasks[0].p, sizeof(Task) * cap), "alloc") &&
               ck(cudaMalloc(&d_tasks[1].p, sizeof(Task) * 2 * cap), "alloc") &&
               ck(cudaMalloc(&d_bins.p, sizeof(BinStat) * 3 * kBins * (size_t)cap), "alloc") &&
               ck(cudaMalloc(&d_splits.p, sizeof(Split) * cap), "alloc") &&
               ck(cudaMalloc(&d_cursors.p, 8ull * cap), "alloc") && ck(cudaMalloc(&d_child.p, 8ull * cap), "alloc") &&
               ck(cudaMalloc(&d_median.p, sizeof(GBox) * 2 * cap), "alloc");
    };
    if (!ensure_tasks(1024))
        return false;
    if (!ck(cudaMemcpyAsync(d_tasks[0].p, &root, sizeof(Task), cudaMemcpyHostToDevice, s), "upload"))
        return false;
    int counters_h[4] = {1, 0, 0, 0};
    if (!ck(cudaMemcpyAsync(d_counters.p, counters_h, 16, cudaMemcpyHostToDevice, s), "upload"))
        return false;
    int cur = 0;
    int depth = 0;
    for (int level = 0; ntasks > 0; level++) {
        if (level > opt.max_depth + 1) {
            err = "GPU BVH build: depth bound exceeded";
            return false;
        }
        // the next level holds at most 2 tasks per task
        if (2 * ntasks > cap) {
            // grow while keeping the current tasks
            std::vector<Task> keep(ntasks);
            if (!ck(cudaMemcpyAsync(keep.data(), d_tasks[cur].p, sizeof(Task) * ntasks, cudaMemcpyDeviceToHost, s),
                    "download") ||
                !ck(cudaStreamSynchronize(s), "sync"))
                return false;
            if (!ensure_tasks(2 * ntasks))
                return false;
            cur = 0;
            if (!ck(cudaMemcpyAsync(d_tasks[0].p, keep.data(), sizeof(Task) * ntasks, cudaMemcpyHostToDevice, s),
                    "upload"))
                return false;
        }
        Task *tasks = d_tasks[cur].as<Task>();
        Task *next = d_tasks[cur ^ 1].as<Task>();
        k_clear_bins<<<grid_of(3L * kBins * ntasks), 256, 0, s>>>(d_bins.as<BinStat>(), 3 * kBins * ntasks);
        k_bin<<<(n + 255) / 256, 256, 0, s>>>(d_boxes.as<GBox>(), d_cent.as<float4>(), d_idx[0].as<int>(),
                                              d_task_of[0].as<int>(), n, tasks, d_bins.as<BinStat>());
        k_split<<<(ntasks + 127) / 128, 128, 0, s>>>(tasks, ntasks, d_bins.as<BinStat>(), d_splits.as<Split>());
        cudaMemsetAsync(d_cursors.p, 0, 8ull * ntasks, s);
        k_clear_median<<<grid_of(2L * ntasks), 256, 0, s>>>(d_median.as<GBox>(), 2 * ntasks);
        k_partition<<<grid_of(n), 256, 0, s>>>(d_boxes.as<GBox>(), d_cent.as<float4>(), d_idx[0].as<int>(),
                                               d_task_of[0].as<int>(), n, tasks, d_splits.as<Split>(),
                                               d_cursors.as<int>(), d_idx[1].as<int>(), d_side.as<int>(),
                                               d_median.as<GBox>());
        cudaMemsetAsync(d_counters.as<int>() + 1, 0, 4, s);
        k_emit<<<(ntasks + 127) / 128, 128, 0, s>>>(tasks, ntasks, d_splits.as<Split>(), d_median.as<GBox>(),
                                                    d_nodes.as<BVHNode>(), d_counters.as<int>(), next,
                                                    d_child.as<int>(), opt.max_leaf, opt.max_depth,
                                                    d_idx[1].as<int>(), d_boxes.as<GBox>(), d_cent.as<float4>());
        k_retask<<<grid_of(n), 256, 0, s>>>(d_side.as<int>(), d_child.as<int>(), n, d_task_of[1].as<int>());
        std::swap(d_idx[0].p, d_idx[1].p);
        std::swap(d_task_of[0].p, d_task_of[1].p);
        if (!ck(cudaGetLastError(), "launch") ||
            !ck(cudaMemcpyAsync(counters_h, d_counters.p, 16, cudaMemcpyDeviceToHost, s), "download") ||
            !ck(cudaStreamSynchronize(s), "sync"))
            return false;
        ntasks = counters_h[1];
        depth = std::max(depth, counters_h[2]);
        cur ^= 1;
        if (counters_h[0] > max_nodes) {
            err = "GPU BVH build: node bound exceeded";
            return false;
        }
    }
    const int nnodes = counters_h[0];
    out.nodes.resize(nnodes);
    out.order.resize(n);
    out.depth = depth;
    if (!ck(cudaMemcpyAsync(out.nodes.data(), d_nodes.p, sizeof(BVHNode) * nnodes, cudaMemcpyDeviceToHost, s),
            "download") ||
        !ck(cudaMemcpyAsync(out.order.data(), d_idx[0].p, 4ull * n, cudaMemcpyDeviceToHost, s), "download") ||
        !ck(cudaStreamSynchronize(s), "sync"))
        return false;
    return true;
}

}  // namespace vvpt
