// SAH BVH on the GPU (see bvh_gpu.h).
//
// The reference sorts each node's primitives by pMax on every axis, sweeps
// prefix / suffix surface areas and keeps the first split of least cost
// (src/hierarchy/bvh.cpp:5-58). Here every node of one tree level is split
// at once. Three index lists hold the primitives sorted by pMax.x, .y, .z;
// each node owns one contiguous segment [start, end) of all three lists.
// Per level and axis, segmented scans give the prefix and suffix boxes of
// every segment, one thread per position evaluates the reference's cost
// expression (no contraction, the same rounding), and a 64-bit atomicMin of
// (cost, axis, position) per node picks the first least-cost split in the
// reference's loop order. A stable partition of the three lists by side
// keeps every child's lists sorted, so no list is sorted twice. Children
// are contiguous sub-segments, left first, so the final position of a
// primitive is its place in the depth-first leaf order.
#include <cub/cub.cuh>

#include <string>
#include <vector>

#include "bvh_gpu.h"

namespace nr {

namespace {

struct SegBox {
    float lo[3], hi[3];
    int seg;
};

// Segmented union: restarts at every change of segment (segments are
// contiguous, so this is associative).
struct SegUnion {
    __device__ SegBox operator()(const SegBox& a, const SegBox& b) const {
        if (a.seg != b.seg) return b;
        SegBox r;
        r.seg = b.seg;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            r.lo[k] = b.lo[k] < a.lo[k] ? b.lo[k] : a.lo[k];  // std::min
            r.hi[k] = a.hi[k] < b.hi[k] ? b.hi[k] : a.hi[k];  // std::max
        }
        return r;
    }
};

// (d0 d1 + d1 d2 + d2 d0) * 2 in the reference's evaluation order
__device__ __forceinline__ float surface(const SegBox& b) {
    float d0 = __fsub_rn(b.hi[0], b.lo[0]), d1 = __fsub_rn(b.hi[1], b.lo[1]), d2 = __fsub_rn(b.hi[2], b.lo[2]);
    return __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(d0, d1), __fmul_rn(d1, d2)), __fmul_rn(d2, d0)), 2.0f);
}

__device__ __forceinline__ uint32_t order_key(float f) {  // float -> uint32 with the same order
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

struct Nodes {
    int* start;
    int* end;
    int* left;      // child ids, -1 for a leaf
    int* right;
    int* order;     // list whose order a leaf keeps: its parent's split axis, 3 = loader order
    float* box;     // 6 per node
    unsigned long long* key;
    int* mid;
    int* axis;
};

__global__ void k_bounds(const float* __restrict__ pos, int n, float* pmin, float* pmax, uint32_t* keys, int* ids) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = pos + 9 * (size_t)i;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float a = p[k], b = p[3 + k], c = p[6 + k];
        float lo = b < a ? b : a, hi = a < b ? b : a;
        lo = c < lo ? c : lo;
        hi = hi < c ? c : hi;
        pmin[3 * (size_t)i + k] = lo;
        pmax[3 * (size_t)i + k] = hi;
        keys[(size_t)k * n + i] = order_key(hi);
    }
    ids[i] = i;
}

// items of list `list` in forward (rev = 0) or reversed order
__global__ void k_items(const int* __restrict__ list, const int* __restrict__ seg, const float* __restrict__ pmin,
                        const float* __restrict__ pmax, int n, int rev, SegBox* out) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int p = rev ? n - 1 - r : r;
    int t = list[p];
    SegBox b;
#pragma unroll
    for (int k = 0; k < 3; ++k) { b.lo[k] = pmin[3 * (size_t)t + k]; b.hi[k] = pmax[3 * (size_t)t + k]; }
    b.seg = seg[p];
    out[r] = b;
}

// Boxes of the open nodes [n0, n1) and their leaf / split status.
__global__ void k_node_boxes(Nodes N, int n0, int n1, const SegBox* __restrict__ pre) {
    int v = n0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n1) return;
    const SegBox& b = pre[N.end[v] - 1];
    for (int k = 0; k < 3; ++k) { N.box[6 * (size_t)v + k] = b.lo[k]; N.box[6 * (size_t)v + 3 + k] = b.hi[k]; }
    N.key[v] = ~0ull;
    N.left[v] = -1;
    N.right[v] = -1;
}

// Cost of splitting after position p (BVH::_divide's prefix loop).
__global__ void k_costs(Nodes N, int n0, int n1, const int* __restrict__ seg, const SegBox* __restrict__ pre,
                        const SegBox* __restrict__ suf_rev, int n, int axis) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int v = seg[p];
    if (v < n0 || v >= n1) return;
    const int s = N.start[v], size = N.end[v] - s;
    if (size <= 5) return;
    const int i = p - s;
    if (i > size - 2) return;
    const float a = surface(pre[p]);
    const float b = surface(suf_rev[n - 1 - (p + 1)]);
    const float cost = __fadd_rn(__fmul_rn(a, (float)(i + 1)), __fmul_rn(b, (float)(size - i)));
    if (!(cost < 1e38f)) return;  // the reference's start value never loses
    const unsigned long long key = ((unsigned long long)__float_as_uint(cost) << 32) | (unsigned)(axis * size + i);
    atomicMin(&N.key[v], key);
}

__global__ void k_decide(Nodes N, int n0, int n1) {
    int v = n0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n1) return;
    const int size = N.end[v] - N.start[v];
    if (size <= 5) { N.mid[v] = 0; return; }
    unsigned long long k = N.key[v];
    if (k == ~0ull) { N.axis[v] = 0; N.mid[v] = size / 2; return; }  // no finite cost (degenerate input)
    const unsigned low = (unsigned)(k & 0xffffffffu);
    N.axis[v] = (int)(low / (unsigned)size);
    N.mid[v] = (int)(low % (unsigned)size) + 1;
}

__global__ void k_sides(Nodes N, int n0, int n1, const int* __restrict__ seg, const int* const* lists, int n,
                        uint8_t* side) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int v = seg[p];
    if (v < n0 || v >= n1 || N.mid[v] == 0) return;
    int t = lists[N.axis[v]][p];
    side[t] = (p - N.start[v]) >= N.mid[v] ? 1 : 0;
}

__global__ void k_left_flags(Nodes N, int n0, int n1, const int* __restrict__ seg, const int* __restrict__ list,
                             const uint8_t* __restrict__ side, int n, int* flag) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int v = seg[p];
    flag[p] = (v >= n0 && v < n1 && N.mid[v] > 0 && side[list[p]] == 0) ? 1 : 0;
}

// Stable partition of one list inside every split segment: left side first.
__global__ void k_scatter(Nodes N, int n0, int n1, const int* __restrict__ seg, const int* __restrict__ list,
                          const int* __restrict__ ex, const int* __restrict__ flag, int n, int* out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int v = seg[p];
    int q = p;
    if (v >= n0 && v < n1 && N.mid[v] > 0) {
        const int s = N.start[v];
        const int lefts_before = ex[p] - ex[s];
        q = flag[p] ? s + lefts_before : s + N.mid[v] + (p - s - lefts_before);
    }
    out[q] = list[p];
}

__global__ void k_children(Nodes N, int n0, int n1, int* count) {
    int v = n0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n1 || N.mid[v] == 0) return;
    int c = atomicAdd(count, 2);
    const int s = N.start[v], e = N.end[v], m = s + N.mid[v];
    N.start[c] = s; N.end[c] = m; N.order[c] = N.axis[v];
    N.start[c + 1] = m; N.end[c + 1] = e; N.order[c + 1] = N.axis[v];
    N.left[v] = c;
    N.right[v] = c + 1;
}

__global__ void k_reseg(Nodes N, int n0, int n1, int* seg, int n) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int v = seg[p];
    if (v < n0 || v >= n1 || N.mid[v] == 0) return;
    seg[p] = p < N.start[v] + N.mid[v] ? N.left[v] : N.right[v];
}

__global__ void k_final_order(Nodes N, const int* __restrict__ seg, const int* const* lists, int n, int* tri) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int o = N.order[seg[p]];
    tri[p] = o == 3 ? p : lists[o][p];
}

struct Scratch {
    std::vector<void*> ptrs;
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, count * sizeof(T) + 16) != cudaSuccess) throw std::string("out of device memory in BVH build");
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
};

void check(cudaError_t e) {
    if (e != cudaSuccess) throw std::string("CUDA error in BVH build: ") + cudaGetErrorString(e);
}

inline unsigned blocks(long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

std::string build_bvh_gpu(const float* pos_host, int n, Bvh& out, cudaStream_t st, double* device_ms,
                          int depth_limit) {
    out = Bvh{};
    if (n <= 0) return "";
    try {
        Scratch S;
        struct Events {  // destroyed on every way out
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            ~Events() {
                if (e0) cudaEventDestroy(e0);
                if (e1) cudaEventDestroy(e1);
            }
        } ev;
        check(cudaEventCreate(&ev.e0));
        check(cudaEventCreate(&ev.e1));
        cudaEvent_t e0 = ev.e0, e1 = ev.e1;
        float* pos = S.get<float>(9 * (size_t)n);
        check(cudaMemcpyAsync(pos, pos_host, 9 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st));
        check(cudaEventRecord(e0, st));
        float* pmin = S.get<float>(3 * (size_t)n);
        float* pmax = S.get<float>(3 * (size_t)n);
        uint32_t* keys = S.get<uint32_t>(3 * (size_t)n);
        uint32_t* keys_sorted = S.get<uint32_t>((size_t)n);
        int* ids = S.get<int>((size_t)n);
        int* lists[3];
        int* spare[3];
        for (int a = 0; a < 3; ++a) { lists[a] = S.get<int>((size_t)n); spare[a] = S.get<int>((size_t)n); }
        int** lists_dev = S.get<int*>(3);
        int* seg = S.get<int>((size_t)n);
        uint8_t* side = S.get<uint8_t>((size_t)n);
        int* flag = S.get<int>((size_t)n);
        int* ex = S.get<int>((size_t)n);
        SegBox* items = S.get<SegBox>((size_t)n);
        SegBox* pre = S.get<SegBox>((size_t)n);
        SegBox* suf = S.get<SegBox>((size_t)n);
        const size_t cap = 2 * (size_t)n;
        Nodes N;
        N.start = S.get<int>(cap); N.end = S.get<int>(cap); N.left = S.get<int>(cap); N.right = S.get<int>(cap);
        N.order = S.get<int>(cap); N.box = S.get<float>(6 * cap); N.key = S.get<unsigned long long>(cap);
        N.mid = S.get<int>(cap); N.axis = S.get<int>(cap);
        int* count = S.get<int>(1);

        // CUB scratch, sized for the largest of the three operations
        size_t tmp_bytes = 0, b = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, b, keys, keys_sorted, ids, lists[0], n, 0, 32, st);
        tmp_bytes = std::max(tmp_bytes, b);
        cub::DeviceScan::InclusiveScan(nullptr, b, items, pre, SegUnion(), n, st);
        tmp_bytes = std::max(tmp_bytes, b);
        cub::DeviceScan::ExclusiveSum(nullptr, b, flag, ex, n, st);
        tmp_bytes = std::max(tmp_bytes, b);
        void* tmp = S.get<unsigned char>(tmp_bytes);

        k_bounds<<<blocks(n), 256, 0, st>>>(pos, n, pmin, pmax, keys, ids);
        for (int a = 0; a < 3; ++a) {  // stable: equal keys stay in loader order
            b = tmp_bytes;
            check(cub::DeviceRadixSort::SortPairs(tmp, b, keys + (size_t)a * n, keys_sorted, ids, lists[a], n, 0, 32, st));
        }
        check(cudaMemcpyAsync(lists_dev, lists, sizeof(lists), cudaMemcpyHostToDevice, st));
        check(cudaMemsetAsync(seg, 0, (size_t)n * sizeof(int), st));
        const int root_start = 0, root_order = 3;
        check(cudaMemcpyAsync(N.start, &root_start, sizeof(int), cudaMemcpyHostToDevice, st));
        check(cudaMemcpyAsync(N.end, &n, sizeof(int), cudaMemcpyHostToDevice, st));
        check(cudaMemcpyAsync(N.order, &root_order, sizeof(int), cudaMemcpyHostToDevice, st));
        int one = 1;
        check(cudaMemcpyAsync(count, &one, sizeof(int), cudaMemcpyHostToDevice, st));

        int n0 = 0, n1 = 1, levels = 0;
        while (n0 < n1) {
            if (++levels > n + 1) throw std::string("BVH build did not terminate");
            if (levels > depth_limit + 1) {  // the tree would be refused by the traversal's stack
                check(cudaStreamSynchronize(st));  // nothing of the build in flight when its buffers go
                out = Bvh{};
                out.max_depth = depth_limit + 1;
                return "";
            }
            const unsigned nb = blocks(n1 - n0);
            for (int a = 0; a < 3; ++a) {
                k_items<<<blocks(n), 256, 0, st>>>(lists[a], seg, pmin, pmax, n, 0, items);
                b = tmp_bytes;
                check(cub::DeviceScan::InclusiveScan(tmp, b, items, pre, SegUnion(), n, st));
                if (a == 0) k_node_boxes<<<nb, 256, 0, st>>>(N, n0, n1, pre);
                k_items<<<blocks(n), 256, 0, st>>>(lists[a], seg, pmin, pmax, n, 1, items);
                b = tmp_bytes;
                check(cub::DeviceScan::InclusiveScan(tmp, b, items, suf, SegUnion(), n, st));
                k_costs<<<blocks(n), 256, 0, st>>>(N, n0, n1, seg, pre, suf, n, a);
            }
            k_decide<<<nb, 256, 0, st>>>(N, n0, n1);
            k_sides<<<blocks(n), 256, 0, st>>>(N, n0, n1, seg, lists_dev, n, side);
            for (int a = 0; a < 3; ++a) {
                k_left_flags<<<blocks(n), 256, 0, st>>>(N, n0, n1, seg, lists[a], side, n, flag);
                b = tmp_bytes;
                check(cub::DeviceScan::ExclusiveSum(tmp, b, flag, ex, n, st));
                k_scatter<<<blocks(n), 256, 0, st>>>(N, n0, n1, seg, lists[a], ex, flag, n, spare[a]);
                std::swap(lists[a], spare[a]);
            }
            check(cudaMemcpyAsync(lists_dev, lists, sizeof(lists), cudaMemcpyHostToDevice, st));
            k_children<<<nb, 256, 0, st>>>(N, n0, n1, count);
            k_reseg<<<blocks(n), 256, 0, st>>>(N, n0, n1, seg, n);
            int next = 0;
            check(cudaMemcpyAsync(&next, count, sizeof(int), cudaMemcpyDeviceToHost, st));
            check(cudaStreamSynchronize(st));
            n0 = n1;
            n1 = next;
        }
        int* tri = ex;  // reused
        k_final_order<<<blocks(n), 256, 0, st>>>(N, seg, lists_dev, n, tri);
        check(cudaEventRecord(e1, st));
        const int nn = n1;
        std::vector<int> start(nn), end(nn), left(nn), right(nn), leaf_tris(n);
        std::vector<float> box(6 * (size_t)nn);
        check(cudaMemcpyAsync(start.data(), N.start, nn * sizeof(int), cudaMemcpyDeviceToHost, st));
        check(cudaMemcpyAsync(end.data(), N.end, nn * sizeof(int), cudaMemcpyDeviceToHost, st));
        check(cudaMemcpyAsync(left.data(), N.left, nn * sizeof(int), cudaMemcpyDeviceToHost, st));
        check(cudaMemcpyAsync(right.data(), N.right, nn * sizeof(int), cudaMemcpyDeviceToHost, st));
        check(cudaMemcpyAsync(box.data(), N.box, 6 * (size_t)nn * sizeof(float), cudaMemcpyDeviceToHost, st));
        check(cudaMemcpyAsync(leaf_tris.data(), tri, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st));
        check(cudaStreamSynchronize(st));
        check(cudaGetLastError());
        if (device_ms) {
            float ms = 0.f;
            check(cudaEventElapsedTime(&ms, e0, e1));
            *device_ms = ms;
        }

        // depth-first, left child first (the layout build_bvh produces)
        out.nodes.reserve(nn);
        out.leaf_tris = std::move(leaf_tris);
        struct Item { int v, depth, parent, side; };
        std::vector<Item> stack{{0, 0, -1, 0}};
        while (!stack.empty()) {
            Item it = stack.back();
            stack.pop_back();
            const int id = (int)out.nodes.size();
            BvhNode nd;
            for (int k = 0; k < 3; ++k) { nd.lo[k] = box[6 * (size_t)it.v + k]; nd.hi[k] = box[6 * (size_t)it.v + 3 + k]; }
            nd.depth = it.depth;
            if (it.depth > out.max_depth) out.max_depth = it.depth;
            if (left[it.v] < 0) {
                nd.left = nd.right = -1;
                nd.first = start[it.v];
                nd.count = end[it.v] - start[it.v];
            } else {
                nd.left = nd.right = -1;  // filled when the children are emitted
                nd.first = -1;
                nd.count = 0;
                stack.push_back({right[it.v], it.depth + 1, id, 1});
                stack.push_back({left[it.v], it.depth + 1, id, 0});
            }
            out.nodes.push_back(nd);
            if (it.parent >= 0) (it.side ? out.nodes[it.parent].right : out.nodes[it.parent].left) = id;
        }
    } catch (const std::string& e) {
        out = Bvh{};
        return e;
    }
    return "";
}

}  // namespace nr
