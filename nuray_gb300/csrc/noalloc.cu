// nr_intersect_noalloc: closest-hit queries for host arrays without any
// device allocation by the library.
//
// nr_intersect stages host rays and results in device memory it obtains with
// cudaMalloc. Some callers cannot let a library allocate device memory while
// they run: hosts that give a plugin a fixed memory budget at start-up and
// account for every later allocation, or real-time loops that cannot afford
// cudaMalloc's implicit device synchronisation in the middle of a frame.
// For them this entry point stages through one file-scope device array of
// fixed size and calls no cudaMalloc, cudaFree or allocating library
// routine. Under CUDA's lazy module loading the array is reserved on a
// device when the module holding it is first loaded there; the library
// does that, and looks up the array's address, when the first scene is
// created on the device (noalloc_prepare), so the calls themselves load
// and allocate nothing.
#include <mutex>

#include "nr_device.cuh"
#include "noalloc.h"

namespace nr {

namespace {

// Layout of the static scratch: origins and directions (3 floats each), then
// triangle ids, t, b1, b2 (one 32-bit value each), then the error word.
constexpr size_t kOff_o = 0;
constexpr size_t kOff_d = kOff_o + (size_t)NR_NOALLOC_MAX_RAYS * 12;
constexpr size_t kOff_tri = kOff_d + (size_t)NR_NOALLOC_MAX_RAYS * 12;
constexpr size_t kOff_t = kOff_tri + (size_t)NR_NOALLOC_MAX_RAYS * 4;
constexpr size_t kOff_b1 = kOff_t + (size_t)NR_NOALLOC_MAX_RAYS * 4;
constexpr size_t kOff_b2 = kOff_b1 + (size_t)NR_NOALLOC_MAX_RAYS * 4;
constexpr size_t kOff_err = kOff_b2 + (size_t)NR_NOALLOC_MAX_RAYS * 4;
constexpr size_t kScratchBytes = kOff_err + 256;  // 2.6 MB with 65,536 rays
static_assert(kScratchBytes == (size_t)NR_NOALLOC_MAX_RAYS * 40 + 256,
              "the static scratch is sized by include/nuray.h's NR_NOALLOC_MAX_RAYS");

// Held by every device that loads the library until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch per device. The host-side symbol is
// only a stand-in for the device variable, so the address is looked up with
// cudaGetSymbolAddress, once per device, with that device current.
std::mutex g_mu;
void* g_addr[NR_NOALLOC_MAX_DEVICES] = {};

__global__ void k_intersect_noalloc(DeviceScene S, int n, const float* __restrict__ o, const float* __restrict__ d,
                                    int* __restrict__ tri, float* __restrict__ t, float* __restrict__ b1,
                                    float* __restrict__ b2, uint32_t* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float tt, u, v;
    int k = closest_hit(S, mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]), mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]), tt, u, v, err);
    tri[i] = k >= 0 ? __float_as_int(__ldg(&S.tri_geo[3 * k]).w) : -1;
    t[i] = tt;
    b1[i] = u;
    b2[i] = v;
}

// Looks up (once per device, under g_mu) the device address of the scratch
// on the current device, loading its module if lazy loading has not yet.
std::string scratch_address(int device, char** out) {
    if (device < 0 || device >= NR_NOALLOC_MAX_DEVICES) return "device index out of range for the static scratch";
    if (!g_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        g_addr[device] = p;
    }
    *out = static_cast<char*>(g_addr[device]);
    return "";
}

}  // namespace

std::string noalloc_prepare(int device) {
    std::lock_guard<std::mutex> lk(g_mu);
    char* base = nullptr;
    return scratch_address(device, &base);
}

std::string noalloc_intersect(const DeviceScene& S, int device, cudaStream_t st, int n, const float* o, const float* d,
                              int32_t* tri, float* t, float* b1, float* b2) {
    if (n < 0) return "n must be >= 0";
    if (n > NR_NOALLOC_MAX_RAYS)
        return "nr_intersect_noalloc takes at most " + std::to_string(NR_NOALLOC_MAX_RAYS) + " rays per call (got " +
               std::to_string(n) + "); split the batch";
    if (device < 0 || device >= NR_NOALLOC_MAX_DEVICES) return "device index out of range for the static scratch";
    if (n == 0) return "";
    // one call at a time: every call uses the same static array
    std::lock_guard<std::mutex> lk(g_mu);
    // looked up when the scene was created; again here only if that failed
    char* base = nullptr;
    std::string err_addr = scratch_address(device, &base);
    if (!err_addr.empty()) return err_addr;
    float* so = reinterpret_cast<float*>(base + kOff_o);
    float* sd = reinterpret_cast<float*>(base + kOff_d);
    int32_t* stri = reinterpret_cast<int32_t*>(base + kOff_tri);
    float* stt = reinterpret_cast<float*>(base + kOff_t);
    float* sb1 = reinterpret_cast<float*>(base + kOff_b1);
    float* sb2 = reinterpret_cast<float*>(base + kOff_b2);
    uint32_t* serr = reinterpret_cast<uint32_t*>(base + kOff_err);
    const size_t f3 = (size_t)n * 12, f1 = (size_t)n * 4;
    cudaError_t e = cudaSuccess;
    // the array keeps the previous call's contents: the error word starts at zero
    if (e == cudaSuccess) e = cudaMemsetAsync(serr, 0, 4, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(so, o, f3, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sd, d, f3, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return std::string("staging rays: ") + cudaGetErrorString(e);
    k_intersect_noalloc<<<(n + 127) / 128, 128, 0, st>>>(S, n, so, sd, stri, stt, sb1, sb2, serr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return std::string("k_intersect_noalloc: ") + cudaGetErrorString(e);
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(tri, stri, f1, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t, stt, f1, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b1, sb1, f1, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b2, sb2, f1, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, serr, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return std::string("reading results: ") + cudaGetErrorString(e);
    if (err) return "traversal error bits " + std::to_string(err) + " (" + err_bits_text() + ")";
    return "";
}

}  // namespace nr
