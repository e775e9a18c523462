// capi.cu -- host orchestration and C ABI of the GB300 MWU backend (see
// include/hpdex_gb300.h). Resident matrices (CSC or CSR input, int64 or int32 indices),
// plans (a grouping over a matrix) with the batched (CUDA graph, fused p-values) and plain
// launch forms, exact-mode tables, the pipelined one-shot calls that mirror the reference
// binding kernel.mannwhitneyu / kernel.group_mean (AI4Cell/hpdex src/cpp/module.cpp:193-243),
// the serving loop, the no-allocation entry point, BH FDR / fold change, the device memory
// cache and the page-locked result-buffer pool. No CPU fallback: without a usable device
// every entry point fails with HPDEX_ERR_CUDA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/hpdex_gb300.h"
#include "common.cuh"
#include "fdr.cuh"
#include "group_mean.cuh"
#include "mwu_rank.cuh"
#include "pvalue.cuh"
#include "transpose.cuh"
#include "rank_launch.h"

using namespace hpdex;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(expr)                                                                     \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess)                                                             \
            return fail(HPDEX_ERR_CUDA, "CUDA error %s at %s:%d (%s)", cudaGetErrorString(_e), \
                        __FILE__, __LINE__, #expr);                                        \
    } while (0)

#define TRY(expr)                        \
    do {                                 \
        int _s = (expr);                 \
        if (_s != HPDEX_OK) return _s;   \
    } while (0)

constexpr int kRankThreads = 1024;
constexpr int kPlainStreams = 128;  // concurrent streams of the plain form (the device runs at
                                    // most 128 kernels at once)
constexpr int kMeanThreads = 256;

struct DeviceInfo {
    int device = -1;
    int sms = 0;
    size_t smem_per_sm = 0, smem_optin = 0, smem_reserved = 0;
    bool pageable_access = false;
};

// Properties of the current device, queried once per device and process.
int device_info(DeviceInfo& d) {
    static std::mutex mu;
    static std::map<int, DeviceInfo> cache;
    int dev = 0;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return fail(HPDEX_ERR_CUDA, "no CUDA device is available (hpdex_gb300 has no CPU path)");
    CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) { d = it->second; return HPDEX_OK; }
    int v = 0;
    d.device = dev;
    CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev)); d.sms = v;
    CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)); d.smem_per_sm = (size_t)v;
    CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)); d.smem_optin = (size_t)v;
    CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrReservedSharedMemoryPerBlock, dev)); d.smem_reserved = (size_t)v;
    // kernels may read and write pageable host memory directly, through the host's page tables
    // (coherent host memory, as on Grace); not where such access migrates pages on faults
    int ats = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev));
    CUDA_TRY(cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
    d.pageable_access = v != 0 && ats != 0;
    cache[dev] = d;
    return HPDEX_OK;
}

// The p-value stage's erfc table (pvalue.cuh), built once per device and process; *tbl (if
// given) receives its device address, which the rank kernel's fused p-values read. Called
// outside stream capture (it synchronises).
int ensure_erfc_table(const double** tbl = nullptr) {
    static std::mutex mu;
    static std::map<int, const double*> ready;
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (ready[dev]) {
        if (tbl) *tbl = ready[dev];
        return HPDEX_OK;
    }
    void* addr = nullptr;
    CUDA_TRY(cudaGetSymbolAddress(&addr, g_erfc_table));
    cudaStream_t s;
    CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    erfc_table_kernel<<<(kErfcPoints + 255) / 256, 256, 0, s>>>();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) return fail(HPDEX_ERR_CUDA, "erfc table set-up: %s", cudaGetErrorString(e));
    ready[dev] = static_cast<const double*>(addr);
    if (tbl) *tbl = ready[dev];
    return HPDEX_OK;
}

size_t dtype_size(int dt) {
    switch (dt) {
    case HPDEX_INT8: case HPDEX_UINT8: return 1;
    case HPDEX_INT16: case HPDEX_UINT16: return 2;
    case HPDEX_INT32: case HPDEX_UINT32: case HPDEX_FLOAT32: return 4;
    case HPDEX_INT64: case HPDEX_UINT64: case HPDEX_FLOAT64: return 8;
    default: return 0;
    }
}
int key_bytes(int dt) {
    return (dt == HPDEX_INT64 || dt == HPDEX_UINT64 || dt == HPDEX_FLOAT64) ? 8 : 4;
}

// Row ids arrive as int64 (the reference's CscView, sparse.hpp:41-68). Ids outside
// [0, n_rows) are skipped by every kernel, so narrowing maps them to -1.
__global__ void narrow_rows_kernel(const long long* in, int32_t* out, long long n, long long n_rows) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long long r = in[i];
        out[i] = (r >= 0 && r < n_rows) ? (int32_t)r : -1;
    }
}

// Upload of one chunk read straight from the caller's host arrays (systems whose device reaches
// pageable host memory): values copied, row ids narrowed to int32 (-1 outside [0, n_rows)).
// kUploadCTAs CTAs of 1024 threads, four elements in flight per thread, keep the host link busy
// from a few SMs while the persistent rank kernel of the previous chunk holds the others.
constexpr int kUploadCTAs = 24;
template <class V, class R>
__global__ void __launch_bounds__(1024) upload_chunk_kernel(const V* __restrict__ hv, const R* __restrict__ hr,
                                                            V* __restrict__ dv, int32_t* __restrict__ dr,
                                                            long long n, long long n_rows) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    auto narrow = [&](R r) { return ((long long)r >= 0 && (long long)r < n_rows) ? (int32_t)r : -1; };
    for (; i + 3 * stride < n; i += 4 * stride) {
        const V v0 = hv[i], v1 = hv[i + stride], v2 = hv[i + 2 * stride], v3 = hv[i + 3 * stride];
        const R r0 = hr[i], r1 = hr[i + stride], r2 = hr[i + 2 * stride], r3 = hr[i + 3 * stride];
        dv[i] = v0; dv[i + stride] = v1; dv[i + 2 * stride] = v2; dv[i + 3 * stride] = v3;
        dr[i] = narrow(r0); dr[i + stride] = narrow(r1); dr[i + 2 * stride] = narrow(r2); dr[i + 3 * stride] = narrow(r3);
    }
    for (; i < n; i += stride) {
        dv[i] = hv[i];
        dr[i] = narrow(hr[i]);
    }
}

// The same upload with 16-byte accesses: four consecutive entries per thread and step (values and
// row ids as one or two 16-byte words). Host reads over the link reach about 205 GB/s this way
// against 180 GB/s with element-wide loads (GB300, pageable memory; 212 GB/s is the page-locked
// copy rate). Entries [0, lead) and the last (n - lead) % 4 are copied one by one; from `lead`
// on, all four arrays are aligned to their quads (the launcher checks).
template <int B> struct Quad;  // four elements of B bytes
template <> struct Quad<1> { using T = uint32_t; };
template <> struct Quad<2> { using T = uint2; };
template <> struct Quad<4> { using T = uint4; };
template <> struct Quad<8> { struct __align__(16) T { ulonglong2 a, b; }; };

template <class V, class R>
__global__ void __launch_bounds__(1024) upload_chunk_quad_kernel(const V* __restrict__ hv, const R* __restrict__ hr,
                                                                 V* __restrict__ dv, int32_t* __restrict__ dr,
                                                                 long long n, long long n_rows, int lead) {
    using QV = typename Quad<sizeof(V)>::T;
    using QR = typename Quad<sizeof(R)>::T;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    auto narrow = [&](long long r) { return (r >= 0 && r < n_rows) ? (int32_t)r : -1; };
    const long long nq = (n - lead) / 4;
    const long long tail = lead + 4 * nq;
    if (tid < lead) { dv[tid] = hv[tid]; dr[tid] = narrow((long long)hr[tid]); }
    if (tail + tid < n) { dv[tail + tid] = hv[tail + tid]; dr[tail + tid] = narrow((long long)hr[tail + tid]); }
    const QV* qv = reinterpret_cast<const QV*>(hv + lead);
    const QR* qr = reinterpret_cast<const QR*>(hr + lead);
    QV* ov = reinterpret_cast<QV*>(dv + lead);
    int4* orow = reinterpret_cast<int4*>(dr + lead);
    auto rows4 = [&](const QR& w) {
        if constexpr (sizeof(R) == 4)
            return make_int4(narrow((int32_t)w.x), narrow((int32_t)w.y), narrow((int32_t)w.z), narrow((int32_t)w.w));
        else
            return make_int4(narrow((long long)w.a.x), narrow((long long)w.a.y), narrow((long long)w.b.x),
                             narrow((long long)w.b.y));
    };
    long long q = tid;
    for (; q + stride < nq; q += 2 * stride) {  // two quads in flight per thread
        const QV v0 = qv[q], v1 = qv[q + stride];
        const QR r0 = qr[q], r1 = qr[q + stride];
        ov[q] = v0;
        ov[q + stride] = v1;
        orow[q] = rows4(r0);
        orow[q + stride] = rows4(r1);
    }
    if (q < nq) {
        ov[q] = qv[q];
        orow[q] = rows4(qr[q]);
    }
}

// Device memory cache. A released block stays reserved for its device and is handed out
// again to a request of at most its size and at least half of it, so repeated calls (the
// one-shot call allocates a matrix, a plan and their scratch every time) skip cudaMalloc and
// cudaFree. Every entry point returns with its device work complete, so a released block is
// idle. hpdex_release_cached_memory() returns the cached blocks to the driver; an allocation
// that fails does the same for its device and retries once.
class MemCache {
    struct Dev {
        std::multimap<size_t, void*> idle;
        size_t idle_bytes = 0;
    };
    std::mutex mu_;
    std::map<int, Dev> dev_;
    std::map<void*, std::pair<int, size_t>> live_;  // pointer -> device, block size

    static size_t round(size_t b) {
        const size_t g = b >= (size_t(1) << 20) ? (size_t(1) << 20) : 512;
        return (b + g - 1) / g * g;
    }
    void drop_idle(int dev) {  // caller holds mu_
        auto& d = dev_[dev];
        int cur = -1;
        cudaGetDevice(&cur);
        if (cur != dev) cudaSetDevice(dev);
        for (auto& kv : d.idle) cudaFree(kv.second);
        if (cur != dev && cur >= 0) cudaSetDevice(cur);
        d.idle.clear();
        d.idle_bytes = 0;
    }

  public:
    cudaError_t get(void** out, size_t bytes) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        const size_t want = round(bytes);
        {
            std::lock_guard<std::mutex> lock(mu_);
            auto& d = dev_[dev];
            auto it = d.idle.lower_bound(want);
            if (it != d.idle.end() && it->first / 2 <= want) {
                *out = it->second;
                live_[*out] = {dev, it->first};
                d.idle_bytes -= it->first;
                d.idle.erase(it);
                return cudaSuccess;
            }
        }
        e = cudaMalloc(out, want);
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            std::lock_guard<std::mutex> lock(mu_);
            drop_idle(dev);
            e = cudaMalloc(out, want);
        }
        if (e != cudaSuccess) { *out = nullptr; return e; }
        std::lock_guard<std::mutex> lock(mu_);
        live_[*out] = {dev, want};
        return cudaSuccess;
    }
    void put(void* p) {
        if (!p) return;
        std::lock_guard<std::mutex> lock(mu_);
        auto it = live_.find(p);
        if (it == live_.end()) { cudaFree(p); return; }
        auto& d = dev_[it->second.first];
        d.idle.insert({it->second.second, p});
        d.idle_bytes += it->second.second;
        live_.erase(it);
    }
    void release_all() {
        std::lock_guard<std::mutex> lock(mu_);
        for (auto& kv : dev_) drop_idle(kv.first);
    }
};
MemCache& mem_cache() {
    static MemCache* c = new MemCache();  // never destroyed: blocks are released to the driver at exit
    return *c;
}

// Page-locked host buffers for result arrays. The Python wrapper of the one-shot call takes one
// per output array: the device writes the results straight into it, with no pages to fault in
// first, and the buffer comes back when the array is released. A released buffer is handed out
// again to a request of at most its size and at least half of it; at most kHeldBytes are held
// (idle or lent out), beyond which a request gets NULL and the caller uses ordinary memory.
class HostPool {
    std::mutex mu_;
    std::multimap<size_t, void*> idle_;
    std::map<void*, size_t> live_;
    size_t held_ = 0;

  public:
    static constexpr size_t kHeldBytes = size_t(2) << 30;
    void* get(size_t bytes) {
        const size_t g = bytes >= (size_t(32) << 20) ? (size_t(2) << 20) : (size_t(64) << 10);
        const size_t want = (bytes + g - 1) / g * g;
        {
            std::lock_guard<std::mutex> lock(mu_);
            auto it = idle_.lower_bound(want);
            if (it != idle_.end() && it->first / 2 <= want) {
                void* p = it->second;
                live_[p] = it->first;
                idle_.erase(it);
                return p;
            }
            if (held_ + want > kHeldBytes) return nullptr;
            held_ += want;  // reserved while allocating
        }
        void* p = nullptr;
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocPortable | cudaHostAllocMapped);
        void* dp = nullptr;
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&dp, p, 0);
        if (e != cudaSuccess || dp != p) {  // the device must see the buffer at its host address
            cudaGetLastError();
            if (p) cudaFreeHost(p);
            std::lock_guard<std::mutex> lock(mu_);
            held_ -= want;
            return nullptr;
        }
        std::lock_guard<std::mutex> lock(mu_);
        live_[p] = want;
        return p;
    }
    bool put(void* p) {
        std::lock_guard<std::mutex> lock(mu_);
        auto it = live_.find(p);
        if (it == live_.end()) return false;
        idle_.insert({it->second, p});
        live_.erase(it);
        return true;
    }
    void release_idle() {
        std::lock_guard<std::mutex> lock(mu_);
        for (auto& kv : idle_) {
            cudaFreeHost(kv.second);
            held_ -= kv.first;
        }
        idle_.clear();
    }
};
HostPool& host_pool() {
    static HostPool* h = new HostPool();
    return *h;
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DevBuf() { mem_cache().put(p); }
    int alloc(size_t count) {
        if (p) { mem_cache().put(p); p = nullptr; }
        n = count;
        if (count == 0) return HPDEX_OK;
        void* q = nullptr;
        cudaError_t e = mem_cache().get(&q, count * sizeof(T));
        if (e != cudaSuccess) {
            return fail(HPDEX_ERR_CUDA, "device allocation of %zu bytes failed: %s", count * sizeof(T),
                        cudaGetErrorString(e));
        }
        p = static_cast<T*>(q);
        return HPDEX_OK;
    }
};

}  // namespace

// ---------------------------------------------------------------------------------------
struct hpdex_matrix {
    int dtype = 0;
    long long n_rows = 0, n_cols = 0, nnz = 0;
    DevBuf<unsigned char> data;
    DevBuf<int32_t> rows;
    DevBuf<int64_t> indptr;
    DevBuf<unsigned long long> col_kmin, col_kmax;  // per-column key range (resident layout)
    DevBuf<uint32_t> col_has_zero;
    std::vector<long long> col_nnz;  // host copy for scheduling
    long long max_col_nnz = 0;
    bool has_int_cols = true;  // some column stores only small integers (launches then use the
                               // rank kernel with the histogram path)
    DeviceInfo dev;
};

struct hpdex_plan {
    hpdex_matrix* m = nullptr;
    hpdex_mwu_options opt{};
    long long T = 0, G = 0;
    std::vector<long long> group_rows;
    DevBuf<int32_t> gid;
    DevBuf<long long> d_group_rows;
    DevBuf<PConst> d_pconst;  // per-target p-value constants (zero_handling min / max / mix)
    DevBuf<int32_t> order;
    DevBuf<int32_t> queue;
    DevBuf<unsigned long long> err;
    DevBuf<double> U1, P;
    DevBuf<uint32_t> n1, n2;  // zero_handling = none
    // rank scratch: decoded column and bucket-ordered slab, one slice per CTA each
    DevBuf<unsigned char> dk, ek;
    DevBuf<unsigned char> dg, eg;
    DevBuf<unsigned char> gidc;  // group of each row in the rank kernel's group type
    RankTask task{};             // this plan as a rank-kernel task (host copy)
    DevBuf<RankTask> d_task;
    DevBuf<unsigned char> acc;
    DevBuf<uint32_t> cnt;
    RankArgs ra{};
    bool hist_on = true;         // histogram path allowed (hpdex_plan_set_histogram)
    int nbl = 13;                // bucket table of 2^nbl entries (hpdex_plan_set_bucket_bits)
    int cnt_mode = -1;           // run counters: -1 automatic, 1 shared, 0 global memory
                                 // (hpdex_plan_set_run_counters)
    bool fused_pvalues = false;  // asymptotic p-values computed inside the rank kernel
    size_t rank_smem = 0;
    int rank_grid = 0;
    // exact tables
    DevBuf<long long> pair_n1, pair_n2, pair_off, work_off;
    DevBuf<double> tables, pair_recip;
    DevBuf<unsigned long long> work;
    DevBuf<int32_t> pair_of_target, pair_of_test;
    DevBuf<unsigned char> pair_mark;  // zero_handling none: (n1, n2) cells present
    DevBuf<int32_t> pair_index;       //   and their pair ids
    // execution
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int last_launches = 0;
    float last_ms[3] = {0, 0, 0};
    // plain form: concurrent streams for the per-gene launches, fork / join events
    std::vector<cudaStream_t> plain_streams;
    std::vector<cudaEvent_t> plain_join;
    cudaEvent_t plain_fork = nullptr;
    int ensure_plain_streams(int n) {
        if (!plain_fork && cudaEventCreateWithFlags(&plain_fork, cudaEventDisableTiming) != cudaSuccess)
            return fail(HPDEX_ERR_CUDA, "event create failed");
        while ((int)plain_streams.size() < n) {
            cudaStream_t st = nullptr;
            cudaEvent_t ev = nullptr;
            if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
                return fail(HPDEX_ERR_CUDA, "stream create failed");
            plain_streams.push_back(st);
            if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
                return fail(HPDEX_ERR_CUDA, "event create failed");
            plain_join.push_back(ev);
        }
        return HPDEX_OK;
    }
    ~hpdex_plan() {
        for (auto st : plain_streams) cudaStreamDestroy(st);
        for (auto e : plain_join) cudaEventDestroy(e);
        if (plain_fork) cudaEventDestroy(plain_fork);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto& e : ev) if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// ---- dtype dispatch -------------------------------------------------------------------
template <template <class> class F, class... Args>
int dispatch_dtype(int dt, Args&&... args) {
    switch (dt) {
    case HPDEX_INT8: return F<int8_t>::run(args...);
    case HPDEX_UINT8: return F<uint8_t>::run(args...);
    case HPDEX_INT16: return F<int16_t>::run(args...);
    case HPDEX_UINT16: return F<uint16_t>::run(args...);
    case HPDEX_INT32: return F<int32_t>::run(args...);
    case HPDEX_UINT32: return F<uint32_t>::run(args...);
    case HPDEX_INT64: return F<int64_t>::run(args...);
    case HPDEX_UINT64: return F<uint64_t>::run(args...);
    case HPDEX_FLOAT32: return F<float>::run(args...);
    case HPDEX_FLOAT64: return F<double>::run(args...);
    default: return fail(HPDEX_ERR_RUNTIME, "Unsupported dtype for data");
    }
}

int rank_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return HPDEX_OK;
    return fail(HPDEX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

template <class V>
struct KeyRangeLaunch {
    // key ranges of columns [0, w) of indptr (entries ~ a hint for the grid); resets them first
    static int run(const void* data, const int64_t* indptr, long long w, unsigned long long* kmin,
                   unsigned long long* kmax, uint32_t* hz, long long entries, int sms, cudaStream_t s) {
        if (w <= 0) return HPDEX_OK;
        CUDA_TRY(cudaMemsetAsync(kmin, 0xff, sizeof(unsigned long long) * w, s));
        CUDA_TRY(cudaMemsetAsync(kmax, 0, sizeof(unsigned long long) * w, s));
        CUDA_TRY(cudaMemsetAsync(hz, 0, sizeof(uint32_t) * w, s));
        const long long per_block = 8ll * 32 * kRangePer;  // 256 threads
        const int grid = (int)std::max<long long>(1, std::min<long long>((entries + per_block - 1) / per_block, (long long)sms * 16));
        column_key_range_kernel<V><<<grid, 256, 0, s>>>(reinterpret_cast<const V*>(data), indptr, (int32_t)w,
                                                       kmin, kmax, hz);
        CUDA_TRY(cudaGetLastError());
        return HPDEX_OK;
    }
};

template <class V>
struct UploadLaunch {  // one chunk, straight from the host arrays (see upload_chunk_kernel)
    static int run(const void* hv, const int64_t* hr64, const int32_t* hr32, void* dv, int32_t* dr,
                   long long n, long long n_rows, cudaStream_t s) {
        if (n == 0) return HPDEX_OK;
        // quads from the first entry whose device row id is 16-byte aligned, when the other
        // three arrays are aligned to their quads there too (numpy's arrays are, at any chunk
        // start that is a multiple of 4 entries away)
        const int lead = (int)((4 - ((uintptr_t)dr / 4) % 4) % 4);
        auto aligned = [&](const void* p, size_t elem, size_t a) {
            return ((uintptr_t)p + (size_t)lead * elem) % a == 0;
        };
        const size_t qv = std::min<size_t>(16, 4 * sizeof(V));
        const size_t qr = 16;
        const bool quad = n >= lead + 4 && aligned(hv, sizeof(V), qv) && aligned(dv, sizeof(V), qv) &&
                          aligned(hr32 ? (const void*)hr32 : (const void*)hr64, hr32 ? 4 : 8, qr);
        if (quad && hr32)
            upload_chunk_quad_kernel<V, int32_t><<<kUploadCTAs, 1024, 0, s>>>(
                static_cast<const V*>(hv), hr32, static_cast<V*>(dv), dr, n, n_rows, lead);
        else if (quad)
            upload_chunk_quad_kernel<V, int64_t><<<kUploadCTAs, 1024, 0, s>>>(
                static_cast<const V*>(hv), hr64, static_cast<V*>(dv), dr, n, n_rows, lead);
        else if (hr32)
            upload_chunk_kernel<V, int32_t><<<kUploadCTAs, 1024, 0, s>>>(
                static_cast<const V*>(hv), hr32, static_cast<V*>(dv), dr, n, n_rows);
        else
            upload_chunk_kernel<V, int64_t><<<kUploadCTAs, 1024, 0, s>>>(
                static_cast<const V*>(hv), hr64, static_cast<V*>(dv), dr, n, n_rows);
        CUDA_TRY(cudaGetLastError());
        return HPDEX_OK;
    }
};
template <class V>
struct MeanLaunch {
    static int run(const MeanArgs* a, dim3 grid, size_t smem, cudaStream_t s) {
        auto k = group_mean_kernel<V, kMeanThreads>;
        CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kMeanThreads, smem, s>>>(*a);
        CUDA_TRY(cudaGetLastError());
        return HPDEX_OK;
    }
};

// Sets m->has_int_cols from the column flags of the key-range pass: some column with finite
// nonzero values, all of them small integers (bit 1 of col_has_zero clear).
int matrix_int_hint(hpdex_matrix* m) {
    const long long C = m->n_cols;
    m->has_int_cols = false;
    if (C == 0) return HPDEX_OK;
    std::vector<uint32_t> f((size_t)C);
    std::vector<unsigned long long> lo((size_t)C), hi((size_t)C);
    CUDA_TRY(cudaMemcpy(f.data(), m->col_has_zero.p, sizeof(uint32_t) * C, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(lo.data(), m->col_kmin.p, sizeof(unsigned long long) * C, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(hi.data(), m->col_kmax.p, sizeof(unsigned long long) * C, cudaMemcpyDeviceToHost));
    for (long long c = 0; c < C && !m->has_int_cols; ++c)
        m->has_int_cols = !(f[(size_t)c] & 2u) && lo[(size_t)c] <= hi[(size_t)c];
    return HPDEX_OK;
}

// The one-shot call's guess before any column is on the device: integer dtypes may hold small
// integers; float data when its first (up to 4,096) values are finite integers. A wrong guess
// only costs speed: both kernel variants give the same results.
bool host_int_hint(int dtype, const void* data, long long nnz) {
    if (dtype != HPDEX_FLOAT32 && dtype != HPDEX_FLOAT64) return true;
    const long long n = std::min<long long>(nnz, 4096);
    for (long long i = 0; i < n; ++i) {
        const double v = dtype == HPDEX_FLOAT32 ? (double)static_cast<const float*>(data)[i]
                                                : static_cast<const double*>(data)[i];
        if (!(std::fabs(v) < 2147483648.0) || v != std::trunc(v)) return false;
    }
    return n > 0;
}

int validate_csc(const int64_t* indptr, long long n_cols, long long nnz, long long n_rows) {
    if (n_rows < 0 || n_cols < 0 || nnz < 0) return fail(HPDEX_ERR_ARGUMENT, "negative matrix size");
    if (n_rows >= (1ll << 31)) return fail(HPDEX_ERR_UNSUPPORTED, "n_rows must be below 2^31");
    if (n_cols >= (1ll << 31)) return fail(HPDEX_ERR_UNSUPPORTED, "n_cols must be below 2^31");
    for (long long c = 0; c < n_cols; ++c) {
        if (indptr[c] < 0 || indptr[c + 1] < indptr[c] || indptr[c + 1] > nnz)
            return fail(HPDEX_ERR_ARGUMENT,
                        "indptr is not a valid CSC column pointer at column %lld", c);
    }
    return HPDEX_OK;
}

// Row ids: int64 (`indices`, narrowed on the device, ids outside [0, n_rows) marked -1) or
// int32 (`indices32`, copied as they are; every consumer skips ids outside [0, n_rows)).
int upload_matrix(hpdex_matrix* m, const void* data, const int64_t* indices, const int32_t* indices32,
                  const int64_t* indptr) {
    const size_t vs = dtype_size(m->dtype);
    TRY(m->data.alloc(std::max<size_t>(1, (size_t)m->nnz * vs)));
    TRY(m->rows.alloc(std::max<long long>(1, m->nnz)));
    TRY(m->indptr.alloc((size_t)m->n_cols + 1));
    // values and int32 row ids may be host or device memory (hpdex_matrix_create_device)
    if (m->nnz) CUDA_TRY(cudaMemcpy(m->data.p, data, (size_t)m->nnz * vs, cudaMemcpyDefault));
    CUDA_TRY(cudaMemcpy(m->indptr.p, indptr, sizeof(int64_t) * ((size_t)m->n_cols + 1),
                        cudaMemcpyHostToDevice));
    // row ids: int64 -> int32 through a bounded staging buffer
    const long long chunk = 1ll << 24;
    if (m->nnz && indices32) {
        CUDA_TRY(cudaMemcpy(m->rows.p, indices32, sizeof(int32_t) * (size_t)m->nnz, cudaMemcpyDefault));
    } else if (m->nnz) {
        DevBuf<long long> stage;
        TRY(stage.alloc((size_t)std::min(chunk, m->nnz)));
        for (long long off = 0; off < m->nnz; off += chunk) {
            const long long k = std::min(chunk, m->nnz - off);
            CUDA_TRY(cudaMemcpy(stage.p, indices + off, sizeof(long long) * k, cudaMemcpyHostToDevice));
            narrow_rows_kernel<<<(int)std::min<long long>((k + 255) / 256, 8192), 256>>>(
                stage.p, m->rows.p + off, k, m->n_rows);
            CUDA_TRY(cudaGetLastError());
        }
        CUDA_TRY(cudaDeviceSynchronize());
    }
    // per-column key range of finite nonzero values: the bucket function of every plan
    TRY(m->col_kmin.alloc(std::max<long long>(m->n_cols, 1)));
    TRY(m->col_kmax.alloc(std::max<long long>(m->n_cols, 1)));
    TRY(m->col_has_zero.alloc(std::max<long long>(m->n_cols, 1)));
    if (m->n_cols) {
        TRY(dispatch_dtype<KeyRangeLaunch>(m->dtype, (const void*)m->data.p, (const int64_t*)m->indptr.p, m->n_cols,
                                           m->col_kmin.p, m->col_kmax.p, m->col_has_zero.p, m->nnz, m->dev.sms,
                                           (cudaStream_t)0));
        CUDA_TRY(cudaDeviceSynchronize());
    }
    TRY(matrix_int_hint(m));
    m->col_nnz.resize((size_t)m->n_cols);
    m->max_col_nnz = 0;
    for (long long c = 0; c < m->n_cols; ++c) {
        m->col_nnz[(size_t)c] = indptr[c + 1] - indptr[c];
        m->max_col_nnz = std::max(m->max_col_nnz, m->col_nnz[(size_t)c]);
    }
    return HPDEX_OK;
}

// Whether a grouping leaves enough rows out (more than 15 %) for the rank kernel to keep only
// the stored entries in its decoded copy: the slab passes then re-read fewer entries, for the
// cost of one warp-wide atomic per 128 entries in the decoding pass.
int32_t compact_decode(const std::vector<long long>& group_rows, long long n_rows) {
    long long assigned = 0;
    for (long long r : group_rows) assigned += r;
    return (n_rows > 0 && assigned * 100 < n_rows * 85) ? 1 : 0;
}

// The rank-kernel task of a plan: its matrix, grouping and output buffers.
RankTask task_of(const hpdex_matrix* m, const hpdex_plan* p) {
    RankTask t{};
    t.data = m->data.p;
    t.rows = m->rows.p;
    t.indptr = m->indptr.p;
    t.col_kmin = m->col_kmin.p;
    t.col_kmax = m->col_kmax.p;
    t.col_has_zero = m->col_has_zero.p;
    t.n_rows = m->n_rows;
    t.n_cols = (int32_t)m->n_cols;
    t.G = (int32_t)p->G;
    t.group_of_row = p->gidc.p;
    t.zero_handling = p->opt.zero_handling;
    t.tie_correction = p->opt.tie_correction;
    t.group_rows = p->d_group_rows.p;
    t.U1 = p->U1.p;
    t.tie = p->P.p;
    t.n1 = p->n1.p;
    t.n2 = p->n2.p;
    t.err = p->err.p;
    t.alternative = p->opt.alternative;
    t.fast_norm = p->opt.fast_norm;
    t.cc = p->opt.use_continuity ? 0.5 : 0.0;
    t.pconst = p->d_pconst.p;
    t.compact_decode = compact_decode(p->group_rows, m->n_rows);
    return t;
}

// Per-target p-value constants of a grouping (n1 = reference rows, n2 = the target's rows);
// empty under zero_handling none, where n1 and n2 depend on the gene.
std::vector<PConst> target_consts(const std::vector<long long>& group_rows, int zero_handling) {
    std::vector<PConst> k;
    if (zero_handling == HPDEX_ZERO_NONE) return k;
    for (size_t g = 1; g < group_rows.size(); ++g)
        k.push_back(make_pconst((double)group_rows[0], (double)group_rows[g]));
    return k;
}

// Rank-kernel layout for this plan: one 1024-thread CTA per SM; the bucket table takes
// 2^13 entries, then the per-target accumulators, the run counters of as many warps as fit
// (at least 4, else in global memory), and the rest holds a gene's elements when it fits.
// Shared-memory layout, grid and scratch sizes of a rank launch for value type `dtype`,
// layout G and longest column `max_col`.
struct RankLayout {
    int nbl = 13, tie_warps = kRankThreads / 32, acc_in = 1, cnt_in = 1, cap = 0, grid = 0, kb = 4, gb = 2;
    size_t smem = 0;
    long long slice = 0;
    bool need_slab_scratch = false;  // some column exceeds the shared-memory capacity
    size_t dk_bytes() const { return (size_t)grid * slice * kb; }
    size_t dg_bytes() const { return (size_t)grid * slice * gb; }
    size_t acc_bytes(int G) const { return acc_in ? 0 : (size_t)grid * 24 * G; }
    size_t cnt_words(int G) const { return (size_t)grid * tie_warps * ((size_t)RankSmem::cnt_words(G) + G); }
};

// Run counters (per warp, 16 bits per group) stay in shared memory up to this many groups; above
// it they take so much of it (64 KB at 1,024 groups) that the elements' room is worth more: on
// the exact-mode workload (1,501 groups) the counters in global memory, with rounds resolving
// repeated groups by warp match, took the step from 8.01 to 5.51 ms (slabs of 4,600 elements
// became slabs of 18,000).
constexpr int kCountersSharedMaxG = 1024;

// cnt_mode: 1 run counters in shared memory (when the accumulators are), 0 in global memory,
// -1 automatic (kCountersSharedMaxG).
int rank_layout(const DeviceInfo& dev, int dtype, int G, long long max_col, RankLayout* out,
                int nbl = 13, int cnt_mode = -1) {
    RankLayout r;
    r.nbl = nbl;
    r.kb = key_bytes(dtype);
    const size_t budget = std::min(dev.smem_per_sm - dev.smem_reserved, dev.smem_optin) - 2048;
    // accumulators in shared memory when they fit (with the counters, when those are there too);
    // else both in global memory
    r.cnt_in = (cnt_mode == 1 || (cnt_mode < 0 && G <= kCountersSharedMaxG)) ? 1 : 0;
    RankSmem L(r.nbl, G, r.tie_warps, 1, r.cnt_in, 0, r.kb);
    if (L.total + 16384 > budget) {
        r.acc_in = 0;
        r.cnt_in = 0;
        L = RankSmem(r.nbl, G, r.tie_warps, 0, 0, 0, r.kb);
    }
    if (L.total > budget) return fail(HPDEX_ERR_UNSUPPORTED, "rank kernel layout does not fit");
    const size_t left = budget - L.total;
    r.gb = group_bytes(r.acc_in);
    r.cap = (int)std::min<size_t>(left / (r.kb + r.gb + 1), (size_t)1 << 30);  // + big-list entry share
    r.cap = std::max(0, r.cap - 8) & ~7;
    L = RankSmem(r.nbl, G, r.tie_warps, r.acc_in, r.cnt_in, r.cap, r.kb);
    while (L.total > budget && r.cap > 0) {  // the big list is sized for compact slabs
        r.cap = std::max(0, r.cap - 64);
        L = RankSmem(r.nbl, G, r.tie_warps, r.acc_in, r.cnt_in, r.cap, r.kb);
    }
    r.smem = L.total;
    int blocks = 0;
    TRY(rank_status(rank_occupancy(dtype, r.smem, dev.smem_optin, r.acc_in, &blocks), "rank kernel set-up"));
    if (blocks < 1) return fail(HPDEX_ERR_CUDA, "rank kernel does not fit on an SM (smem %zu)", r.smem);
    r.grid = dev.sms * blocks;
    // whole 128-byte lines per CTA slice (vector access, L2 discards)
    r.slice = rank_slice(max_col);
    r.need_slab_scratch = (long long)r.cap < max_col;
    *out = r;
    return HPDEX_OK;
}

// Fills the launch-wide fields of RankArgs (layout and scratch) from a layout.
void set_layout_args(RankArgs& a, const RankLayout& r, int G, void* dk, void* dg, void* ek, void* eg,
                     unsigned char* acc, uint32_t* cnt) {
    a.G = G;
    a.dk_global = dk;
    a.dg_global = dg;
    a.ek_global = ek;
    a.eg_global = eg;
    a.slice = r.slice;
    a.acc_global = acc;
    a.cnt_global = cnt;
    a.nb_max_log2 = r.nbl;
    a.elem_smem_cap = r.cap;
    a.acc_in_smem = r.acc_in;
    a.cnt_in_smem = r.cnt_in;
    a.tie_warps = r.tie_warps;
}

int configure_rank(hpdex_plan* p) {
    const hpdex_matrix* m = p->m;
    const int G = (int)p->G;
    RankLayout r;
    TRY(rank_layout(m->dev, m->dtype, G, m->max_col_nnz, &r, p->nbl, p->cnt_mode));
    p->rank_smem = r.smem;
    p->rank_grid = r.grid;
    TRY(p->dk.alloc(r.dk_bytes()));
    TRY(p->dg.alloc(r.dg_bytes()));
    if (r.need_slab_scratch) {
        TRY(p->ek.alloc(r.dk_bytes()));
        TRY(p->eg.alloc(r.dg_bytes()));
    }
    TRY(p->gidc.alloc((size_t)std::max<long long>(m->n_rows, 1) * r.gb));
    if (!r.acc_in) TRY(p->acc.alloc(r.acc_bytes(G)));
    TRY(p->cnt.alloc(r.cnt_words(G)));

    RankTask& t = p->task;
    t = task_of(m, p);
    TRY(p->d_task.alloc(1));
    CUDA_TRY(cudaMemcpy(p->d_task.p, &t, sizeof(RankTask), cudaMemcpyHostToDevice));
    RankArgs& a = p->ra;
    a.tasks = p->d_task.p;
    a.order = p->order.p;
    a.order_task = nullptr;
    a.n_order = (int32_t)m->n_cols;
    a.queue = p->queue.p;
    a.single_gene = -1;
    a.no_histogram = (p->hist_on && m->has_int_cols) ? 0 : 1;
    a.any_compact = t.compact_decode;
    set_layout_args(a, r, G, p->dk.p, p->dg.p, p->ek.p, p->eg.p, p->acc.p, p->cnt.p);
    return HPDEX_OK;
}

int launch_pvalues_asymptotic(hpdex_plan* p, cudaStream_t s) {
    PArgs a{};
    a.U1 = p->U1.p;
    a.P = p->P.p;
    a.n = p->T * p->m->n_cols;
    a.n_cols = (int32_t)p->m->n_cols;
    a.col_lo = 0;
    a.col_w = (int32_t)p->m->n_cols;
    a.group_rows = p->d_group_rows.p;
    a.n1g = p->n1.p;
    a.n2t = p->n2.p;
    a.pk = p->d_pconst.p;
    a.zero_handling = p->opt.zero_handling;
    a.alternative = p->opt.alternative;
    a.cc = p->opt.use_continuity ? 0.5 : 0.0;
    a.fast = p->opt.fast_norm;
    if (a.n == 0) return HPDEX_OK;
    const int grid = (int)std::min<long long>((a.n + 255) / 256, (long long)p->m->dev.sms * 8);
    mwu_pvalue_asymptotic_kernel<<<grid, 256, 0, s>>>(a);
    CUDA_TRY(cudaGetLastError());
    return HPDEX_OK;
}

// Builds the exact tables for the distinct (n1, n2) of this plan and launches the lookup.
int run_exact(hpdex_plan* p, cudaStream_t s) {
    const long long C = p->m->n_cols, T = p->T, n = T * C;
    if (n == 0) return HPDEX_OK;
    std::map<std::pair<long long, long long>, int> pairs;
    std::vector<int32_t> pot;  // pair of target / test
    // zero_handling none, sizes in a small dense map: the device marks the (n1, n2) cells that
    // occur and looks the pair of each test up in a dense index (no per-test host work)
    long long H = 0, W = 0;
    if (p->opt.zero_handling == HPDEX_ZERO_NONE) {
        H = p->group_rows[0] + 1;
        for (long long t = 1; t <= T; ++t) W = std::max(W, p->group_rows[(size_t)t] + 1);
    }
    const bool dense_pairs = p->opt.zero_handling == HPDEX_ZERO_NONE && H * W <= (1ll << 22);
    std::vector<int32_t> hidx;
    if (dense_pairs) {
        TRY(p->pair_mark.alloc((size_t)(H * W)));
        CUDA_TRY(cudaMemsetAsync(p->pair_mark.p, 0, (size_t)(H * W), s));
        const int g = (int)std::min<long long>((n + 255) / 256, (long long)p->m->dev.sms * 8);
        exact_mark_pairs_kernel<<<g, 256, 0, s>>>(p->n1.p, p->n2.p, n, (int32_t)C, (int32_t)H,
                                                  (int32_t)W, p->pair_mark.p);
        CUDA_TRY(cudaGetLastError());
        std::vector<unsigned char> mark((size_t)(H * W));
        CUDA_TRY(cudaMemcpyAsync(mark.data(), p->pair_mark.p, mark.size(), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        hidx.assign((size_t)(H * W), -1);
        for (long long r = 0; r < H * W; ++r)
            if (mark[(size_t)r]) {
                const int id = (int)pairs.size();
                pairs.emplace(std::make_pair(r / W, r % W), id);
                hidx[(size_t)r] = id;
            }
    } else if (p->opt.zero_handling == HPDEX_ZERO_NONE) {
        std::vector<uint32_t> h1((size_t)C), h2((size_t)n);
        CUDA_TRY(cudaStreamSynchronize(s));
        CUDA_TRY(cudaMemcpy(h1.data(), p->n1.p, sizeof(uint32_t) * C, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(h2.data(), p->n2.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
        pot.resize((size_t)n);
        for (long long i = 0; i < n; ++i) {
            const long long c = i % C;
            auto key = std::make_pair((long long)h1[(size_t)c], (long long)h2[(size_t)i]);
            auto it = pairs.find(key);
            if (it == pairs.end()) it = pairs.emplace(key, (int)pairs.size()).first;
            pot[(size_t)i] = it->second;
        }
    } else {
        pot.resize((size_t)T);
        for (long long t = 0; t < T; ++t) {
            auto key = std::make_pair(p->group_rows[0], p->group_rows[(size_t)t + 1]);
            auto it = pairs.find(key);
            if (it == pairs.end()) it = pairs.emplace(key, (int)pairs.size()).first;
            pot[(size_t)t] = it->second;
        }
    }
    const int np = (int)pairs.size();
    std::vector<long long> hn1(np), hn2(np), hoff(np), hwoff(np);
    long long tot = 0, wtot = 0;
    for (auto& kv : pairs) {
        const int i = kv.second;
        hn1[i] = kv.first.first;
        hn2[i] = kv.first.second;
        const long long umax = hn1[i] * hn2[i];
        if (umax > (1ll << 26))
            return fail(HPDEX_ERR_UNSUPPORTED,
                        "method='exact': n1*n2 = %lld exceeds the exact-table limit 2^26", umax);
        hoff[i] = tot;
        tot += 2 * (umax + 1);
        hwoff[i] = wtot;
        const long long mside = std::min(hn1[i], hn2[i]);
        const long long w = p->opt.exact_variant == HPDEX_EXACT_MWU_NULL ? (mside + 1) * (umax + 1)
                                                                        : 2 * (umax + 1);
        if (w > (1ll << 28))
            return fail(HPDEX_ERR_UNSUPPORTED, "method='exact': table work space too large");
        wtot += w;
    }
    TRY(p->pair_n1.alloc(np));
    TRY(p->pair_n2.alloc(np));
    TRY(p->pair_off.alloc(np));
    TRY(p->work_off.alloc(np));
    TRY(p->tables.alloc((size_t)std::max<long long>(tot, 1)));
    TRY(p->work.alloc((size_t)std::max<long long>(wtot, 1)));
    CUDA_TRY(cudaMemcpyAsync(p->pair_n1.p, hn1.data(), sizeof(long long) * np, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(p->pair_n2.p, hn2.data(), sizeof(long long) * np, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(p->pair_off.p, hoff.data(), sizeof(long long) * np, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(p->work_off.p, hwoff.data(), sizeof(long long) * np, cudaMemcpyHostToDevice, s));
    DevBuf<int32_t>& pmap = (p->opt.zero_handling == HPDEX_ZERO_NONE) ? p->pair_of_test : p->pair_of_target;
    if (!pot.empty()) {
        TRY(pmap.alloc(pot.size()));
        CUDA_TRY(cudaMemcpyAsync(pmap.p, pot.data(), sizeof(int32_t) * pot.size(), cudaMemcpyHostToDevice, s));
    }
    if (dense_pairs) {
        TRY(p->pair_index.alloc(hidx.size()));
        CUDA_TRY(cudaMemcpyAsync(p->pair_index.p, hidx.data(), sizeof(int32_t) * hidx.size(),
                                 cudaMemcpyHostToDevice, s));
    }
    ExactTables et{};
    et.pair_n1 = p->pair_n1.p;
    et.pair_n2 = p->pair_n2.p;
    et.offset = p->pair_off.p;
    et.tables = p->tables.p;
    et.work = p->work.p;
    et.work_off = p->work_off.p;
    et.n_pairs = np;
    et.variant = p->opt.exact_variant;
    if (np > 0) {
        if (p->opt.exact_variant == HPDEX_EXACT_MWU_NULL)
            exact_null_table_kernel<256><<<np, 256, 0, s>>>(et);
        else
            exact_reference_table_kernel<256><<<np, 256, 0, s>>>(et);
        CUDA_TRY(cudaGetLastError());
        TRY(p->pair_recip.alloc((size_t)np));
        exact_recip_kernel<<<(np + 255) / 256, 256, 0, s>>>(p->pair_n1.p, p->pair_n2.p, p->pair_off.p,
                                                            p->tables.p, np, p->pair_recip.p);
        CUDA_TRY(cudaGetLastError());
    }
    ExactArgs a{};
    a.U1 = p->U1.p;
    a.P = p->P.p;
    a.n = n;
    a.n_cols = (int32_t)C;
    a.group_rows = p->d_group_rows.p;
    a.n1g = p->n1.p;
    a.n2t = p->n2.p;
    a.zero_handling = p->opt.zero_handling;
    a.alternative = p->opt.alternative;
    a.variant = p->opt.exact_variant;
    a.pair_of_target = p->pair_of_target.p;
    a.pair_of_test = p->pair_of_test.p;
    a.pair_index = dense_pairs ? p->pair_index.p : nullptr;
    a.pair_w = (int32_t)W;
    a.pair_h = (int32_t)H;
    a.pair_n1 = p->pair_n1.p;
    a.pair_n2 = p->pair_n2.p;
    a.offset = p->pair_off.p;
    a.tables = p->tables.p;
    a.recip = p->pair_recip.p;
    const int grid = (int)std::min<long long>((n + 255) / 256, (long long)p->m->dev.sms * 8);
    mwu_pvalue_exact_kernel<<<grid, 256, 0, s>>>(a);
    CUDA_TRY(cudaGetLastError());
    return HPDEX_OK;
}

// The status and message of a run's device error words (reference wording: the lowest
// (column, group) wins, as in the single-threaded reference).
int decode_errors(const unsigned long long* e, long long G_, std::string* msg) {
    const unsigned long long G = (unsigned long long)G_;
    char buf[256];
    if (e[0] != ~0ull) {
        const unsigned long long c = e[0] / G, g = e[0] % G;
        if (g == 0) snprintf(buf, sizeof buf, "Sample too small for reference at column %llu", c);
        else snprintf(buf, sizeof buf, "Sample too small for group %llu at column %llu", g, c);
        *msg = buf;
        return HPDEX_ERR_RUNTIME;
    }
    if (e[1] != ~0ull) {
        const unsigned long long c = e[1] / G, g = e[1] % G;
        snprintf(buf, sizeof buf,
                 "column %llu stores more entries for group %llu than the group has rows "
                 "(duplicate row indices)", c, g);
        *msg = buf;
        return HPDEX_ERR_ARGUMENT;
    }
    return HPDEX_OK;
}

int check_device_errors(hpdex_plan* p) {
    unsigned long long e[kErrWords];
    CUDA_TRY(cudaMemcpy(e, p->err.p, sizeof e, cudaMemcpyDeviceToHost));
    std::string msg;
    const int st = decode_errors(e, p->G, &msg);
    if (st != HPDEX_OK) return fail(st, "%s", msg.c_str());
    return HPDEX_OK;
}

// Rank kernel(s) for one run; batched = persistent + queue, plain = one launch per gene.
int enqueue_rank(hpdex_plan* p, int mode, cudaStream_t s, int* launches) {
    if (p->m->n_cols == 0) return HPDEX_OK;
    // group ids in the rank kernel's type (16-bit when its accumulators are in shared memory)
    {
        const long long R = p->m->n_rows;
        const int grid = (int)std::max<long long>(1, std::min<long long>((R + 255) / 256, (long long)p->m->dev.sms * 8));
        if (p->ra.acc_in_smem)
            prepare_group_ids_kernel<uint16_t><<<grid, 256, 0, s>>>(p->gid.p, R, (int32_t)p->G, reinterpret_cast<uint16_t*>(p->gidc.p));
        else
            prepare_group_ids_kernel<uint32_t><<<grid, 256, 0, s>>>(p->gid.p, R, (int32_t)p->G, reinterpret_cast<uint32_t*>(p->gidc.p));
        CUDA_TRY(cudaGetLastError());
        *launches += 1;
    }
    if (mode == HPDEX_MODE_BATCHED) {
        CUDA_TRY(cudaMemsetAsync(p->queue.p, 0, sizeof(int32_t), s));
        p->ra.single_gene = -1;
        TRY(rank_status(rank_launch(p->m->dtype, p->ra, p->rank_grid, p->rank_smem, s), "rank kernel launch"));
        *launches += 1;
    } else {
        // plain form: one single-CTA launch per gene, in column order, no queue and no graph;
        // the launches go round-robin to concurrent streams (each on its own scratch slice) so
        // that they fill the GPU as far as independent launches can
        const int ns = std::max(1, std::min(p->rank_grid, kPlainStreams));
        TRY(p->ensure_plain_streams(ns));
        CUDA_TRY(cudaEventRecord(p->plain_fork, s));
        for (int k = 0; k < ns; ++k) CUDA_TRY(cudaStreamWaitEvent(p->plain_streams[k], p->plain_fork, 0));
        int st = HPDEX_OK;
        for (long long c = 0; c < p->m->n_cols && st == HPDEX_OK; ++c) {
            const int k = (int)(c % ns);
            p->ra.single_gene = (int32_t)c;
            p->ra.cta_base = k;
            st = rank_status(rank_launch(p->m->dtype, p->ra, 1, p->rank_smem, p->plain_streams[k]),
                             "rank kernel launch");
            if (st == HPDEX_OK) *launches += 1;
        }
        p->ra.single_gene = -1;
        p->ra.cta_base = 0;
        for (int k = 0; k < ns; ++k) {  // join (also after a failed launch)
            CUDA_TRY(cudaEventRecord(p->plain_join[k], p->plain_streams[k]));
            CUDA_TRY(cudaStreamWaitEvent(s, p->plain_join[k], 0));
        }
        TRY(st);
    }
    return HPDEX_OK;
}

// Device transpose of a cells x genes CSR into the resident CSC layout (transpose.cuh).
template <class V>
struct TransposeLaunch {
    template <class GI>  // gene ids: int64, or int32 (scipy's index type) uploaded as they are
    static int run(hpdex_matrix* m, const void* h_data, const GI* h_genes, const int64_t* h_rowptr) {
        const long long R = m->n_rows, C = m->n_cols, nnz_in = m->nnz;
        const size_t vs = sizeof(V);
        DevBuf<unsigned char> dval;
        DevBuf<GI> dgen;
        DevBuf<int64_t> dptr, col_total;
        DevBuf<uint32_t> cnt;
        TRY(dval.alloc(std::max<size_t>(1, (size_t)nnz_in * vs)));
        TRY(dgen.alloc(std::max<long long>(1, nnz_in)));
        TRY(dptr.alloc((size_t)R + 1));
        TRY(col_total.alloc(std::max<long long>(C, 1)));
        if (nnz_in) {
            CUDA_TRY(cudaMemcpy(dval.p, h_data, (size_t)nnz_in * vs, cudaMemcpyHostToDevice));
            CUDA_TRY(cudaMemcpy(dgen.p, h_genes, sizeof(GI) * nnz_in, cudaMemcpyHostToDevice));
        }
        CUDA_TRY(cudaMemcpy(dptr.p, h_rowptr, sizeof(int64_t) * (R + 1), cudaMemcpyHostToDevice));
        TRY(m->indptr.alloc((size_t)C + 1));
        const long long nb0 = std::max<long long>(1, std::min<long long>(R, (long long)m->dev.sms * 4));
        const long long rpb = std::max<long long>(1, (R + nb0 - 1) / nb0);
        const int nb = (int)std::max<long long>(1, (R + rpb - 1) / rpb);
        TRY(cnt.alloc((size_t)nb * std::max<long long>(C, 1)));
        const size_t smem = sizeof(uint32_t) * (size_t)C;
        const bool in_smem = smem <= 160 * 1024;
        if (in_smem) {
            CUDA_TRY(cudaFuncSetAttribute(csr_block_count_kernel<true, GI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            CUDA_TRY(cudaFuncSetAttribute(csr_scatter_kernel<V, true, GI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            csr_block_count_kernel<true, GI><<<nb, kTransposeThreads, smem>>>(dptr.p, dgen.p, R, rpb, (int)C, cnt.p);
        } else {
            CUDA_TRY(cudaMemset(cnt.p, 0, sizeof(uint32_t) * (size_t)nb * C));
            csr_block_count_kernel<false, GI><<<nb, kTransposeThreads>>>(dptr.p, dgen.p, R, rpb, (int)C, cnt.p);
        }
        CUDA_TRY(cudaGetLastError());
        if (C) {
            csr_column_scan_kernel<<<(int)((C + 255) / 256), 256>>>(cnt.p, nb, (int)C, col_total.p);
            column_pointer_scan_kernel<<<1, 1024>>>(col_total.p, (int)C, m->indptr.p);
            CUDA_TRY(cudaGetLastError());
        } else {
            CUDA_TRY(cudaMemset(m->indptr.p, 0, sizeof(int64_t)));
        }
        std::vector<int64_t> ip((size_t)C + 1);
        CUDA_TRY(cudaMemcpy(ip.data(), m->indptr.p, sizeof(int64_t) * (C + 1), cudaMemcpyDeviceToHost));
        m->nnz = ip[(size_t)C];  // entries with a gene id outside [0, C) are dropped
        TRY(m->data.alloc(std::max<size_t>(1, (size_t)m->nnz * vs)));
        TRY(m->rows.alloc(std::max<long long>(1, m->nnz)));
        if (in_smem)
            csr_scatter_kernel<V, true, GI><<<nb, kTransposeThreads, smem>>>(dptr.p, dgen.p, reinterpret_cast<const V*>(dval.p), R, rpb,
                                                                       (int)C, cnt.p, m->indptr.p, m->rows.p,
                                                                       reinterpret_cast<V*>(m->data.p));
        else
            csr_scatter_kernel<V, false, GI><<<nb, kTransposeThreads>>>(dptr.p, dgen.p, reinterpret_cast<const V*>(dval.p), R, rpb,
                                                                  (int)C, cnt.p, m->indptr.p, m->rows.p,
                                                                  reinterpret_cast<V*>(m->data.p));
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaDeviceSynchronize());
        m->col_nnz.resize((size_t)C);
        m->max_col_nnz = 0;
        for (long long c = 0; c < C; ++c) {
            m->col_nnz[(size_t)c] = ip[(size_t)c + 1] - ip[(size_t)c];
            m->max_col_nnz = std::max(m->max_col_nnz, m->col_nnz[(size_t)c]);
        }
        return HPDEX_OK;
    }
};

int oneshot_pipelined(int32_t dtype, const void* data, const int64_t* indices, const int32_t* indices32,
                      const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                      const int32_t* group_id, int64_t n_targets, const hpdex_mwu_options* opt,
                      double* U1_out, double* P_out);
int matrix_group_mean(const hpdex_matrix* m, const int32_t* group_id, int64_t n_groups,
                      int32_t include_zeros, double* out);
int plan_create(hpdex_matrix* m, const int32_t* group_id, int64_t n_targets,
                const hpdex_mwu_options* opt, hpdex_plan** out, bool lpt_order);

}  // namespace

// =======================================================================================
extern "C" {

void hpdex_mwu_options_default(hpdex_mwu_options* o) {
    if (!o) return;
    o->ref_sorted = 0;
    o->tar_sorted = 0;
    o->tie_correction = 1;
    o->use_continuity = 0;
    o->fast_norm = 0;
    o->zero_handling = HPDEX_ZERO_NONE;
    o->alternative = HPDEX_TWO_SIDED;
    o->method = HPDEX_ASYMPTOTIC;
    o->exact_variant = HPDEX_EXACT_REFERENCE;
}

const char* hpdex_last_error(void) { return g_last_error.c_str(); }

int hpdex_selftest_erfc(int64_t n_points, double* max_rel_err, double* max_abs_err) {
    if (n_points < 1 || !max_rel_err || !max_abs_err) return fail(HPDEX_ERR_ARGUMENT, "bad arguments");
    DeviceInfo dev;
    TRY(device_info(dev));
    TRY(ensure_erfc_table());
    DevBuf<unsigned long long> out;
    TRY(out.alloc(2));
    CUDA_TRY(cudaMemset(out.p, 0, 2 * sizeof(unsigned long long)));
    const int grid = (int)std::min<long long>((n_points + 255) / 256, (long long)dev.sms * 8);
    erfc_check_kernel<<<grid, 256>>>(n_points, out.p, out.p + 1);
    CUDA_TRY(cudaGetLastError());
    unsigned long long h[2];
    CUDA_TRY(cudaMemcpy(h, out.p, sizeof h, cudaMemcpyDeviceToHost));
    std::memcpy(max_rel_err, &h[0], sizeof(double));
    std::memcpy(max_abs_err, &h[1], sizeof(double));
    return HPDEX_OK;
}

int hpdex_selftest_erfc_values(const double* x, int64_t n, double* out) {
    if (n < 0 || (n > 0 && (!x || !out))) return fail(HPDEX_ERR_ARGUMENT, "bad arguments");
    DeviceInfo dev;
    TRY(device_info(dev));
    TRY(ensure_erfc_table());
    if (n == 0) return HPDEX_OK;
    DevBuf<double> buf;
    TRY(buf.alloc(2 * (size_t)n));
    CUDA_TRY(cudaMemcpy(buf.p, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    const int grid = (int)std::min<long long>((n + 255) / 256, (long long)dev.sms * 8);
    erfc_values_kernel<<<grid, 256>>>(buf.p, n, buf.p + n);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpy(out, buf.p + n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    return HPDEX_OK;
}

int hpdex_selftest_division(int64_t n_cases, uint64_t seed, int64_t* mismatches) {
    if (n_cases < 0 || !mismatches) return fail(HPDEX_ERR_ARGUMENT, "bad arguments");
    DeviceInfo dev;
    TRY(device_info(dev));
    DevBuf<unsigned long long> out;
    TRY(out.alloc(1));
    CUDA_TRY(cudaMemset(out.p, 0, sizeof(unsigned long long)));
    if (n_cases) {
        const int grid = (int)std::min<long long>((n_cases + 255) / 256, (long long)dev.sms * 16);
        division_check_kernel<<<grid, 256>>>(n_cases, seed, out.p);
        CUDA_TRY(cudaGetLastError());
    }
    unsigned long long h = 0;
    CUDA_TRY(cudaMemcpy(&h, out.p, sizeof h, cudaMemcpyDeviceToHost));
    *mismatches = (int64_t)h;
    return HPDEX_OK;
}

int hpdex_bh_fdr(const double* p, int64_t n, double* fdr) {
    if (n < 0 || (n > 0 && (!p || !fdr))) return fail(HPDEX_ERR_ARGUMENT, "bad arguments");
    if (n <= 1) {
        if (n == 1) {
            if (!(p[0] >= 0.0 && p[0] <= 1.0)) return fail(HPDEX_ERR_ARGUMENT, "All values in `ps` must lie between 0. and 1.");
            fdr[0] = p[0];
        }
        return HPDEX_OK;
    }
    if (n >= (1ll << 31)) return fail(HPDEX_ERR_UNSUPPORTED, "at most 2^31 - 1 p-values");
    DeviceInfo dev;
    TRY(device_info(dev));
    const int nb = (int)((n + kSortTile - 1) / kSortTile);
    DevBuf<unsigned long long> k0, k1;
    DevBuf<uint32_t> v0, v1, counts, bad;
    DevBuf<double> agg, carry, out;
    TRY(k0.alloc((size_t)n));
    TRY(k1.alloc((size_t)n));
    TRY(v0.alloc((size_t)n));
    TRY(v1.alloc((size_t)n));
    TRY(counts.alloc((size_t)256 * nb));
    TRY(bad.alloc(1));
    TRY(agg.alloc((size_t)nb));
    TRY(carry.alloc((size_t)nb));
    TRY(out.alloc((size_t)n));
    cudaStream_t s = 0;
    CUDA_TRY(cudaMemcpyAsync(k0.p, p, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemsetAsync(bad.p, 0, sizeof(uint32_t), s));
    canonical_zero_kernel<<<std::min(nb, dev.sms * 8), 256, 0, s>>>(k0.p, n);
    unsigned long long* kin = k0.p;
    unsigned long long* kout = k1.p;
    uint32_t* vin = nullptr;
    uint32_t* vout = v1.p;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 8 * pass;
        radix_count_kernel<<<nb, kSortThreads, 0, s>>>(kin, n, shift, counts.p, nb);
        radix_scan_kernel<<<1, 1024, 0, s>>>(counts.p, (long long)256 * nb);
        radix_scatter_kernel<<<nb, kSortThreads, 0, s>>>(kin, vin, kout, vout, n, shift, counts.p, nb);
        CUDA_TRY(cudaGetLastError());
        std::swap(kin, kout);
        vin = vout;
        vout = (vout == v1.p) ? v0.p : v1.p;
    }
    bh_block_min_kernel<<<nb, kSortThreads, 0, s>>>(kin, n, agg.p, bad.p);
    bh_carry_kernel<<<1, 1024, 0, s>>>(agg.p, nb, carry.p);
    bh_apply_kernel<<<nb, kSortThreads, 0, s>>>(kin, vin, n, carry.p, out.p);
    CUDA_TRY(cudaGetLastError());
    uint32_t bad_h = 0;
    CUDA_TRY(cudaMemcpyAsync(&bad_h, bad.p, sizeof bad_h, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    if (bad_h) return fail(HPDEX_ERR_ARGUMENT, "All values in `ps` must lie between 0. and 1.");
    CUDA_TRY(cudaMemcpy(fdr, out.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return HPDEX_OK;
}

int hpdex_fold_change(const double* means, int64_t n_genes, int64_t n_groups, double clip,
                      double* fold, double* log2fold) {
    if (n_genes < 0 || n_groups < 1 || !means || !fold || !log2fold) return fail(HPDEX_ERR_ARGUMENT, "bad arguments");
    const long long n = (n_groups - 1) * n_genes;
    if (n == 0) return HPDEX_OK;
    DeviceInfo dev;
    TRY(device_info(dev));
    DevBuf<double> dm, df, dl;
    TRY(dm.alloc((size_t)(n_genes * n_groups)));
    TRY(df.alloc((size_t)n));
    TRY(dl.alloc((size_t)n));
    CUDA_TRY(cudaMemcpy(dm.p, means, sizeof(double) * n_genes * n_groups, cudaMemcpyHostToDevice));
    const int grid = (int)std::min<long long>((n + 255) / 256, (long long)dev.sms * 8);
    fold_change_kernel<<<grid, 256>>>(dm.p, n_genes, (int)n_groups, clip, df.p, dl.p);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpy(fold, df.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(log2fold, dl.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return HPDEX_OK;
}

int hpdex_release_cached_memory(void) {
    mem_cache().release_all();
    host_pool().release_idle();
    return HPDEX_OK;
}

int hpdex_host_buffer_acquire(int64_t bytes, void** ptr) {
    if (!ptr || bytes < 0) return fail(HPDEX_ERR_ARGUMENT, "bad arguments");
    *ptr = bytes > 0 ? host_pool().get((size_t)bytes) : nullptr;
    return HPDEX_OK;
}

int hpdex_host_buffer_release(void* ptr) {
    if (!ptr) return HPDEX_OK;
    if (!host_pool().put(ptr)) return fail(HPDEX_ERR_ARGUMENT, "not a buffer of hpdex_host_buffer_acquire");
    return HPDEX_OK;
}

int hpdex_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int hpdex_device_sm_count(int32_t* sms) {
    if (!sms) return fail(HPDEX_ERR_ARGUMENT, "sms is NULL");
    DeviceInfo dev;
    TRY(device_info(dev));
    *sms = dev.sms;
    return HPDEX_OK;
}

namespace {
int matrix_create(int32_t dtype, const void* data, const int64_t* indices, const int32_t* indices32,
                  const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz, hpdex_matrix** out) {
    if (!out) return fail(HPDEX_ERR_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (dtype_size(dtype) == 0) return fail(HPDEX_ERR_RUNTIME, "Unsupported dtype for data");
    if (!indptr || (nnz > 0 && (!data || (!indices && !indices32)))) return fail(HPDEX_ERR_ARGUMENT, "NULL matrix pointer");
    TRY(validate_csc(indptr, n_cols, nnz, n_rows));
    hpdex_matrix* m = new hpdex_matrix();
    m->dtype = dtype;
    m->n_rows = n_rows;
    m->n_cols = n_cols;
    m->nnz = nnz;
    int st = device_info(m->dev);
    if (st == HPDEX_OK) st = upload_matrix(m, data, indices, indices32, indptr);
    if (st != HPDEX_OK) { delete m; return st; }
    *out = m;
    return HPDEX_OK;
}
}  // namespace

int hpdex_matrix_create(int32_t dtype, const void* data, const int64_t* indices,
                        const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                        hpdex_matrix** out) {
    return matrix_create(dtype, data, indices, nullptr, indptr, n_rows, n_cols, nnz, out);
}

int hpdex_matrix_create_idx32(int32_t dtype, const void* data, const int32_t* indices,
                              const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                              hpdex_matrix** out) {
    return matrix_create(dtype, data, nullptr, indices, indptr, n_rows, n_cols, nnz, out);
}

int hpdex_matrix_create_device(int32_t dtype, const void* d_data, const int32_t* d_rows,
                               const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                               hpdex_matrix** out) {
    return matrix_create(dtype, d_data, nullptr, d_rows, indptr, n_rows, n_cols, nnz, out);
}

int hpdex_matrix_destroy(hpdex_matrix* m) {
    delete m;
    return HPDEX_OK;
}

int hpdex_matrix_info(const hpdex_matrix* m, int64_t* n_rows, int64_t* n_cols, int64_t* nnz,
                      int64_t* device_bytes) {
    if (!m) return fail(HPDEX_ERR_ARGUMENT, "matrix is NULL");
    if (n_rows) *n_rows = m->n_rows;
    if (n_cols) *n_cols = m->n_cols;
    if (nnz) *nnz = m->nnz;
    if (device_bytes)
        *device_bytes = (int64_t)(m->data.n + m->rows.n * 4 + m->indptr.n * 8);
    return HPDEX_OK;
}

int hpdex_plan_create(hpdex_matrix* m, const int32_t* group_id, int64_t n_targets,
                      const hpdex_mwu_options* opt, hpdex_plan** out) {
    return plan_create(m, group_id, n_targets, opt, out, true);
}

}  // extern "C"

namespace {
// lpt_order: fill the work queue's gene order (longest first) here; the pipelined one-shot
// call writes its own per-chunk order instead
int plan_create(hpdex_matrix* m, const int32_t* group_id, int64_t n_targets,
                const hpdex_mwu_options* opt, hpdex_plan** out, bool lpt_order) {
    if (!out) return fail(HPDEX_ERR_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!m || !opt) return fail(HPDEX_ERR_ARGUMENT, "NULL matrix or options");
    if (n_targets < 1) return fail(HPDEX_ERR_RUNTIME, "[mannwhitney] n_targets must be >= 1 (>=1 target groups)");
    if (m->n_rows > 0 && !group_id) return fail(HPDEX_ERR_ARGUMENT, "group_id is NULL");
    if (opt->zero_handling < 0 || opt->zero_handling > 3) return fail(HPDEX_ERR_ARGUMENT, "zero_handling must be 0..3");
    if (opt->alternative < 0 || opt->alternative > 2) return fail(HPDEX_ERR_ARGUMENT, "alternative must be 0..2");
    if (opt->method != HPDEX_EXACT && opt->method != HPDEX_ASYMPTOTIC) return fail(HPDEX_ERR_ARGUMENT, "method must be 1 (exact) or 2 (asymptotic)");
    if (n_targets >= (1ll << 30)) return fail(HPDEX_ERR_UNSUPPORTED, "n_targets too large");
    std::unique_ptr<hpdex_plan> p(new hpdex_plan());
    p->m = m;
    p->opt = *opt;
    p->T = n_targets;
    p->G = n_targets + 1;
    const long long C = m->n_cols, R = m->n_rows, G = p->G;
    p->group_rows.assign((size_t)G, 0);
    for (long long r = 0; r < R; ++r) {
        const int g = group_id[r];
        if (g >= 0 && g < G) ++p->group_rows[(size_t)g];
    }
    // reference-style errors raised before any launch (mannwhitneyu.cpp:967-1020: for
    // min/max/mix the sample sizes are the group sizes, identical for every column)
    if (opt->zero_handling != HPDEX_ZERO_NONE && C > 0) {
        if (p->group_rows[0] < 2) return fail(HPDEX_ERR_RUNTIME, "Sample too small for reference at column 0");
        for (long long g = 1; g < G; ++g)
            if (p->group_rows[(size_t)g] < 2)
                return fail(HPDEX_ERR_RUNTIME, "Sample too small for group %lld at column 0", g);
    }
    CUDA_TRY(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    for (auto& e : p->ev) CUDA_TRY(cudaEventCreate(&e));
    TRY(p->gid.alloc(std::max<long long>(R, 1)));
    if (R) CUDA_TRY(cudaMemcpy(p->gid.p, group_id, sizeof(int32_t) * R, cudaMemcpyHostToDevice));
    TRY(p->d_group_rows.alloc((size_t)G));
    CUDA_TRY(cudaMemcpy(p->d_group_rows.p, p->group_rows.data(), sizeof(long long) * G, cudaMemcpyHostToDevice));
    {
        const std::vector<PConst> k = target_consts(p->group_rows, opt->zero_handling);
        if (!k.empty()) {
            TRY(p->d_pconst.alloc(k.size()));
            CUDA_TRY(cudaMemcpy(p->d_pconst.p, k.data(), sizeof(PConst) * k.size(), cudaMemcpyHostToDevice));
        }
    }
    // longest genes first: the work queue hands them out before the short tail
    TRY(p->order.alloc(std::max<long long>(C, 1)));
    if (lpt_order && C) {
        std::vector<int32_t> order((size_t)C);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
            return m->col_nnz[(size_t)a] > m->col_nnz[(size_t)b];
        });
        CUDA_TRY(cudaMemcpy(p->order.p, order.data(), sizeof(int32_t) * C, cudaMemcpyHostToDevice));
    }
    TRY(p->queue.alloc(1));
    TRY(p->err.alloc(kErrWords));
    const size_t n = (size_t)(p->T * C);
    TRY(p->U1.alloc(std::max<size_t>(n, 1)));
    TRY(p->P.alloc(std::max<size_t>(n, 1)));
    if (opt->zero_handling == HPDEX_ZERO_NONE) {
        TRY(p->n1.alloc(std::max<long long>(C, 1)));
        TRY(p->n2.alloc(std::max<size_t>(n, 1)));
    }
    TRY(configure_rank(p.get()));
    const double* tbl = nullptr;
    TRY(ensure_erfc_table(&tbl));
    if (opt->method == HPDEX_ASYMPTOTIC) {  // p-values inside the rank kernel by default
        p->fused_pvalues = true;
        p->ra.erfc_table = tbl;
    }
    *out = p.release();
    return HPDEX_OK;
}

}  // namespace

extern "C" {

int hpdex_plan_destroy(hpdex_plan* p) {
    delete p;
    return HPDEX_OK;
}

int hpdex_plan_run(hpdex_plan* p, int32_t mode) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    if (mode != HPDEX_MODE_BATCHED && mode != HPDEX_MODE_PLAIN) return fail(HPDEX_ERR_ARGUMENT, "mode must be 0 or 1");
    cudaStream_t s = p->stream;
    int launches = 0;
    const bool exact = p->opt.method == HPDEX_EXACT;
    if (mode == HPDEX_MODE_BATCHED && !exact) {
        if (!p->graph_exec) {
            // capture: error-word reset, queue reset, rank kernel, p-value kernel
            CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int st = HPDEX_OK;
            int l = 0;
            // event-record nodes (a plain record under capture only adds a dependency)
            const unsigned ext = cudaEventRecordExternal;
            if (cudaEventRecordWithFlags(p->ev[0], s, ext) != cudaSuccess) st = fail(HPDEX_ERR_CUDA, "event record failed");
            if (st == HPDEX_OK && cudaMemsetAsync(p->err.p, 0xff, kErrWords * sizeof(unsigned long long), s) != cudaSuccess)
                st = fail(HPDEX_ERR_CUDA, "memset failed");
            if (st == HPDEX_OK) st = enqueue_rank(p, mode, s, &l);
            if (st == HPDEX_OK && cudaEventRecordWithFlags(p->ev[1], s, ext) != cudaSuccess) st = fail(HPDEX_ERR_CUDA, "event record failed");
            if (st == HPDEX_OK && !p->fused_pvalues) st = launch_pvalues_asymptotic(p, s);
            if (st == HPDEX_OK && cudaEventRecordWithFlags(p->ev[2], s, ext) != cudaSuccess) st = fail(HPDEX_ERR_CUDA, "event record failed");
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (st != HPDEX_OK) { if (g) cudaGraphDestroy(g); return st; }
            if (ce != cudaSuccess) return fail(HPDEX_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
            p->graph = g;
            CUDA_TRY(cudaGraphInstantiate(&p->graph_exec, g, 0));
        }
        CUDA_TRY(cudaGraphLaunch(p->graph_exec, s));
        launches = (p->m->n_cols > 0 ? 2 : 0) + (!p->fused_pvalues && p->T * p->m->n_cols > 0 ? 1 : 0);
    } else {
        CUDA_TRY(cudaEventRecord(p->ev[0], s));
        CUDA_TRY(cudaMemsetAsync(p->err.p, 0xff, kErrWords * sizeof(unsigned long long), s));
        TRY(enqueue_rank(p, mode, s, &launches));
        CUDA_TRY(cudaEventRecord(p->ev[1], s));
        if (exact) {
            TRY(run_exact(p, s));
            launches += 2;
        } else if (!p->fused_pvalues) {
            TRY(launch_pvalues_asymptotic(p, s));
            launches += 1;
        }
        CUDA_TRY(cudaEventRecord(p->ev[2], s));
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    p->last_launches = launches;
    CUDA_TRY(cudaEventElapsedTime(&p->last_ms[0], p->ev[0], p->ev[2]));
    CUDA_TRY(cudaEventElapsedTime(&p->last_ms[1], p->ev[0], p->ev[1]));
    CUDA_TRY(cudaEventElapsedTime(&p->last_ms[2], p->ev[1], p->ev[2]));
    return check_device_errors(p);
}

int hpdex_plan_autotune(hpdex_plan* p, int32_t reps, int32_t* run_counters_out,
                        int32_t* bucket_bits_out, float* ms_out) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    if (reps < 1) return fail(HPDEX_ERR_ARGUMENT, "reps must be >= 1");
    // candidate layouts: run counters in shared / global memory x bucket table 2^13 / 2^12; each
    // gives the same results, so the fastest (mean CUDA-event time of `reps` batched runs after
    // one untimed run) is kept
    const int32_t modes[2] = {1, 0}, bits[2] = {13, 12};
    const int32_t old_mode = p->cnt_mode, old_bits = p->nbl;
    float best = 0.0f;
    int32_t best_mode = 1, best_bits = 13;
    int st = HPDEX_OK;
    for (int k = 0; k < 4 && st == HPDEX_OK; ++k) {
        st = hpdex_plan_set_run_counters(p, modes[k / 2]);
        if (st == HPDEX_OK) st = hpdex_plan_set_bucket_bits(p, bits[k % 2]);
        if (st == HPDEX_OK) st = hpdex_plan_run(p, HPDEX_MODE_BATCHED);
        float total = 0.0f;
        for (int r = 0; r < reps && st == HPDEX_OK; ++r) {
            st = hpdex_plan_run(p, HPDEX_MODE_BATCHED);
            total += p->last_ms[0];
        }
        if (st != HPDEX_OK) break;
        const float ms = total / (float)reps;
        if (ms_out) ms_out[k] = ms;
        if (k == 0 || ms < best) {
            best = ms;
            best_mode = modes[k / 2];
            best_bits = bits[k % 2];
        }
    }
    if (st != HPDEX_OK) {  // the plan keeps the layout it had (the error stays the one reported)
        const std::string msg = hpdex_last_error();
        hpdex_plan_set_run_counters(p, old_mode);
        hpdex_plan_set_bucket_bits(p, old_bits);
        return fail(st, "%s", msg.c_str());
    }
    TRY(hpdex_plan_set_run_counters(p, best_mode));
    TRY(hpdex_plan_set_bucket_bits(p, best_bits));
    if (run_counters_out) *run_counters_out = best_mode;
    if (bucket_bits_out) *bucket_bits_out = best_bits;
    return HPDEX_OK;
}

int hpdex_plan_set_fused_pvalues(hpdex_plan* p, int32_t on) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    if (p->opt.method != HPDEX_ASYMPTOTIC) {
        if (on) return fail(HPDEX_ERR_UNSUPPORTED, "fused p-values need method=asymptotic");
        return HPDEX_OK;
    }
    const double* tbl = nullptr;
    TRY(ensure_erfc_table(&tbl));
    const bool f = on != 0;
    if (f == p->fused_pvalues) return HPDEX_OK;
    p->fused_pvalues = f;
    p->ra.erfc_table = f ? tbl : nullptr;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }  // re-captured
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    return HPDEX_OK;
}

int hpdex_plan_set_bucket_bits(hpdex_plan* p, int32_t bits) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    if (bits < 9 || bits > 13) return fail(HPDEX_ERR_ARGUMENT, "bucket bits must be in [9, 13]");
    if (bits == p->nbl) return HPDEX_OK;
    const int old = p->nbl;
    const RankArgs keep = p->ra;  // the plan's other launch settings stay as they were
    p->nbl = bits;
    int st = configure_rank(p);
    if (st != HPDEX_OK) {
        p->nbl = old;
        configure_rank(p);
    }
    p->ra.erfc_table = keep.erfc_table;
    p->ra.drain_wait = keep.drain_wait;
    p->ra.no_histogram = keep.no_histogram;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }  // re-captured
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    return st;
}

int hpdex_plan_set_run_counters(hpdex_plan* p, int32_t mode) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    if (mode < -1 || mode > 1) return fail(HPDEX_ERR_ARGUMENT, "run counter mode must be -1, 0 or 1");
    if (mode == p->cnt_mode) return HPDEX_OK;
    const int old = p->cnt_mode;
    const RankArgs keep = p->ra;  // the plan's other launch settings stay as they were
    p->cnt_mode = mode;
    int st = configure_rank(p);
    if (st != HPDEX_OK) {
        p->cnt_mode = old;
        configure_rank(p);
    }
    p->ra.erfc_table = keep.erfc_table;
    p->ra.drain_wait = keep.drain_wait;
    p->ra.no_histogram = keep.no_histogram;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }  // re-captured
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    return st;
}

int hpdex_plan_set_histogram(hpdex_plan* p, int32_t on) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    p->hist_on = on != 0;
    const int32_t off = (p->hist_on && p->m->has_int_cols) ? 0 : 1;
    if (p->ra.no_histogram == off) return HPDEX_OK;
    p->ra.no_histogram = off;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }  // re-captured
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    return HPDEX_OK;
}

int hpdex_plan_set_drain_wait(hpdex_plan* p, int32_t on) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    const int32_t w = on ? 1 : 0;
    if (p->ra.drain_wait == w) return HPDEX_OK;
    p->ra.drain_wait = w;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }  // re-captured
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    return HPDEX_OK;
}

int hpdex_plan_download(hpdex_plan* p, double* U1_out, double* P_out) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    const size_t n = (size_t)(p->T * p->m->n_cols);
    if (n == 0) return HPDEX_OK;
    if (U1_out) CUDA_TRY(cudaMemcpy(U1_out, p->U1.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    if (P_out) CUDA_TRY(cudaMemcpy(P_out, p->P.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    return HPDEX_OK;
}

int hpdex_plan_timings(const hpdex_plan* p, float* ms3, int32_t* launches) {
    if (!p) return fail(HPDEX_ERR_ARGUMENT, "plan is NULL");
    if (ms3) { ms3[0] = p->last_ms[0]; ms3[1] = p->last_ms[1]; ms3[2] = p->last_ms[2]; }
    if (launches) *launches = p->last_launches;
    return HPDEX_OK;
}

int hpdex_mannwhitneyu(int32_t dtype, const void* data, const int64_t* indices,
                       const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                       const int32_t* group_id, int64_t n_targets,
                       const hpdex_mwu_options* opt, int32_t threads, double* U1_out,
                       double* P_out) {
    (void)threads;
    if (!opt) return fail(HPDEX_ERR_ARGUMENT, "options are NULL");
    if (n_targets < 1) return fail(HPDEX_ERR_RUNTIME, "[mannwhitney] n_targets must be >= 1 (>=1 target groups)");
    if (opt->method != HPDEX_EXACT)
        return oneshot_pipelined(dtype, data, indices, nullptr, indptr, n_rows, n_cols, nnz, group_id, n_targets,
                                 opt, U1_out, P_out);
    hpdex_matrix* m = nullptr;
    TRY(hpdex_matrix_create(dtype, data, indices, indptr, n_rows, n_cols, nnz, &m));
    hpdex_plan* p = nullptr;
    int st = hpdex_plan_create(m, group_id, n_targets, opt, &p);
    if (st == HPDEX_OK) st = hpdex_plan_run(p, HPDEX_MODE_BATCHED);
    if (st == HPDEX_OK) st = hpdex_plan_download(p, U1_out, P_out);
    hpdex_plan_destroy(p);
    hpdex_matrix_destroy(m);
    return st;
}

int hpdex_mannwhitneyu_idx32(int32_t dtype, const void* data, const int32_t* indices,
                             const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                             const int32_t* group_id, int64_t n_targets,
                             const hpdex_mwu_options* opt, int32_t threads, double* U1_out,
                             double* P_out) {
    if (!opt) return fail(HPDEX_ERR_ARGUMENT, "options are NULL");
    if (n_targets < 1) return fail(HPDEX_ERR_RUNTIME, "[mannwhitney] n_targets must be >= 1 (>=1 target groups)");
    if (nnz < 0) return fail(HPDEX_ERR_ARGUMENT, "nnz must be >= 0");
    if (opt->method != HPDEX_EXACT)
        return oneshot_pipelined(dtype, data, nullptr, indices, indptr, n_rows, n_cols, nnz, group_id, n_targets,
                                 opt, U1_out, P_out);
    // exact p-values: through the int64 path
    if (nnz > 0 && !indices) return fail(HPDEX_ERR_ARGUMENT, "NULL matrix pointer");
    std::vector<int64_t> wide((size_t)nnz);
    for (int64_t i = 0; i < nnz; ++i) wide[(size_t)i] = indices[i];
    return hpdex_mannwhitneyu(dtype, data, wide.data(), indptr, n_rows, n_cols, nnz, group_id, n_targets, opt,
                              threads, U1_out, P_out);
}

int hpdex_group_mean(int32_t dtype, const void* data, const int64_t* indices,
                     const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                     const int32_t* group_id, int64_t n_groups, int32_t include_zeros,
                     int32_t use_kahan, int32_t threads, double* out) {
    (void)threads;
    (void)use_kahan;
    if (n_groups <= 0 || n_cols <= 0) return HPDEX_OK;  // the reference returns an empty result
    if (n_groups >= (1ll << 30)) return fail(HPDEX_ERR_UNSUPPORTED, "n_groups too large");
    hpdex_matrix* m = nullptr;
    TRY(hpdex_matrix_create(dtype, data, indices, indptr, n_rows, n_cols, nnz, &m));
    std::unique_ptr<hpdex_matrix> hold(m);
    return matrix_group_mean(m, group_id, n_groups, include_zeros, out);
}

int hpdex_matrix_group_mean(const hpdex_matrix* m, const int32_t* group_id, int64_t n_groups,
                            int32_t include_zeros, double* out) {
    if (!m) return fail(HPDEX_ERR_ARGUMENT, "matrix is NULL");
    if (n_groups <= 0 || m->n_cols <= 0) return HPDEX_OK;
    if (n_groups >= (1ll << 30)) return fail(HPDEX_ERR_UNSUPPORTED, "n_groups too large");
    return matrix_group_mean(m, group_id, n_groups, include_zeros, out);
}

}  // extern "C"
namespace {
template <class GI>
int matrix_create_csr(int32_t dtype, const void* data, const GI* indices, const int64_t* indptr,
                      int64_t n_rows, int64_t n_cols, int64_t nnz, hpdex_matrix** out) {
    if (!out) return fail(HPDEX_ERR_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (dtype_size(dtype) == 0) return fail(HPDEX_ERR_RUNTIME, "Unsupported dtype for data");
    if (!indptr || (nnz > 0 && (!data || !indices))) return fail(HPDEX_ERR_ARGUMENT, "NULL matrix pointer");
    if (n_rows < 0 || n_cols < 0 || nnz < 0) return fail(HPDEX_ERR_ARGUMENT, "negative matrix size");
    if (n_rows >= (1ll << 31) || n_cols >= (1ll << 31)) return fail(HPDEX_ERR_UNSUPPORTED, "n_rows and n_cols must be below 2^31");
    for (long long r = 0; r < n_rows; ++r)
        if (indptr[r] < 0 || indptr[r + 1] < indptr[r] || indptr[r + 1] > nnz)
            return fail(HPDEX_ERR_ARGUMENT, "indptr is not a valid CSR row pointer at row %lld", r);
    std::unique_ptr<hpdex_matrix> m(new hpdex_matrix());
    m->dtype = dtype;
    m->n_rows = n_rows;
    m->n_cols = n_cols;
    m->nnz = nnz;
    TRY(device_info(m->dev));
    TRY(dispatch_dtype<TransposeLaunch>(dtype, m.get(), data, indices, indptr));
    TRY(m->col_kmin.alloc(std::max<long long>(n_cols, 1)));
    TRY(m->col_kmax.alloc(std::max<long long>(n_cols, 1)));
    TRY(m->col_has_zero.alloc(std::max<long long>(n_cols, 1)));
    if (n_cols) {
        TRY(dispatch_dtype<KeyRangeLaunch>(dtype, (const void*)m->data.p, (const int64_t*)m->indptr.p, m->n_cols,
                                           m->col_kmin.p, m->col_kmax.p, m->col_has_zero.p, m->nnz, m->dev.sms,
                                           (cudaStream_t)0));
        CUDA_TRY(cudaDeviceSynchronize());
    }
    TRY(matrix_int_hint(m.get()));
    *out = m.release();
    return HPDEX_OK;
}
}  // namespace
extern "C" {

int hpdex_matrix_create_csr(int32_t dtype, const void* data, const int64_t* indices,
                            const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                            hpdex_matrix** out) {
    return matrix_create_csr(dtype, data, indices, indptr, n_rows, n_cols, nnz, out);
}

int hpdex_matrix_create_csr_idx32(int32_t dtype, const void* data, const int32_t* indices,
                                  const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                                  hpdex_matrix** out) {
    return matrix_create_csr(dtype, data, indices, indptr, n_rows, n_cols, nnz, out);
}

}  // extern "C"

// =======================================================================================
// Group means of a resident matrix (reference group_mean_core, mannwhitneyu.cpp:1118-1192).
// =======================================================================================
namespace {
int matrix_group_mean(const hpdex_matrix* m, const int32_t* group_id, int64_t n_groups,
                      int32_t include_zeros, double* out) {
    const long long n_rows = m->n_rows, n_cols = m->n_cols;
    if (n_rows > 0 && !group_id) return fail(HPDEX_ERR_ARGUMENT, "group_id is NULL");
    std::vector<long long> rows_per((size_t)n_groups, 0);
    for (long long r = 0; r < n_rows; ++r) {
        const int g = group_id[r];
        if (g >= 0 && g < n_groups) ++rows_per[(size_t)g];
    }
    DevBuf<int32_t> gid;
    DevBuf<long long> grows;
    DevBuf<double> dout;
    DevBuf<unsigned char> acc;
    TRY(gid.alloc(std::max<long long>(n_rows, 1)));
    TRY(grows.alloc((size_t)n_groups));
    TRY(dout.alloc((size_t)(n_cols * n_groups)));
    if (n_rows) CUDA_TRY(cudaMemcpy(gid.p, group_id, sizeof(int32_t) * n_rows, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(grows.p, rows_per.data(), sizeof(long long) * n_groups, cudaMemcpyHostToDevice));
    MeanArgs a{};
    a.data = m->data.p;
    a.rows = m->rows.p;
    a.indptr = m->indptr.p;
    a.n_rows = n_rows;
    a.n_cols = (int32_t)n_cols;
    a.G = (int32_t)n_groups;
    a.gid = gid.p;
    a.group_rows = grows.p;
    a.include_zeros = include_zeros;
    a.out = dout.p;
    const size_t need = (size_t)n_groups * 16;
    const size_t budget = std::min(m->dev.smem_optin, m->dev.smem_per_sm / 2);
    const int grid = (int)std::min<long long>(n_cols, (long long)m->dev.sms * 4);
    size_t smem = 0;
    if (need <= budget) {
        a.acc_in_smem = 1;
        smem = need;
    } else {
        a.acc_in_smem = 0;
        TRY(acc.alloc((size_t)grid * need));
        a.acc_global = acc.p;
    }
    TRY(dispatch_dtype<MeanLaunch>(m->dtype, &a, dim3(grid), smem, (cudaStream_t)0));
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaMemcpy(out, dout.p, sizeof(double) * n_cols * n_groups, cudaMemcpyDeviceToHost));
    return HPDEX_OK;
}
}  // namespace

// =======================================================================================
// Pipelined one-shot call (asymptotic method).
//
// hpdex_mannwhitneyu receives the matrix in host memory. The columns are cut into chunks of
// about equal nnz; a copy stream moves chunk k+1 (values, and int64 row ids into one of two
// staging buffers) while the compute stream narrows the row ids of chunk k, computes its
// column key ranges, ranks its genes (the persistent rank kernel over the chunk's genes,
// longest first) and finishes its p-values. When the device can access pageable host
// memory the p-value kernel writes U1 and P straight into the caller's arrays; otherwise
// they are copied back at the end. Host<->device traffic is the bound of this call, so the
// kernels run in the shadow of the copies except for the last chunk.
// =======================================================================================
namespace {

constexpr int kPipelineChunks = 12;
constexpr int kComputeStreams = 2;  // chunks alternate between this many compute streams

// Row ids come as int64 (`indices`, narrowed on the device through staging buffers) or as
// int32 (`indices32`, uploaded straight into the matrix: half the bytes; ids outside
// [0, n_rows) are skipped by the rank kernel as the narrowing would mark them).
int oneshot_pipelined(int32_t dtype, const void* data, const int64_t* indices, const int32_t* indices32,
                      const int64_t* indptr, int64_t n_rows, int64_t n_cols, int64_t nnz,
                      const int32_t* group_id, int64_t n_targets, const hpdex_mwu_options* opt,
                      double* U1_out, double* P_out) {
    const size_t vs = dtype_size(dtype);
    if (vs == 0) return fail(HPDEX_ERR_RUNTIME, "Unsupported dtype for data");
    const bool idx32 = indices32 != nullptr;
    if (!indptr || (nnz > 0 && (!data || (!indices && !indices32)))) return fail(HPDEX_ERR_ARGUMENT, "NULL matrix pointer");
    TRY(validate_csc(indptr, n_cols, nnz, n_rows));
    const long long C = n_cols;

    // matrix shell: device buffers and host metadata; the entries arrive chunk by chunk
    std::unique_ptr<hpdex_matrix> m(new hpdex_matrix());
    m->dtype = dtype;
    m->n_rows = n_rows;
    m->n_cols = n_cols;
    m->nnz = nnz;
    TRY(device_info(m->dev));
    TRY(m->data.alloc(std::max<size_t>(1, (size_t)nnz * vs)));
    TRY(m->rows.alloc(std::max<long long>(1, nnz)));
    TRY(m->indptr.alloc((size_t)C + 1));
    TRY(m->col_kmin.alloc(std::max<long long>(C, 1)));
    TRY(m->col_kmax.alloc(std::max<long long>(C, 1)));
    TRY(m->col_has_zero.alloc(std::max<long long>(C, 1)));
    m->col_nnz.resize((size_t)C);
    for (long long c = 0; c < C; ++c) {
        m->col_nnz[(size_t)c] = indptr[c + 1] - indptr[c];
        m->max_col_nnz = std::max(m->max_col_nnz, m->col_nnz[(size_t)c]);
    }
    m->has_int_cols = host_int_hint(dtype, data, nnz);
    if (C == 0) {
        CUDA_TRY(cudaMemcpy(m->indptr.p, indptr, sizeof(int64_t), cudaMemcpyHostToDevice));
        hpdex_plan* praw = nullptr;
        TRY(plan_create(m.get(), group_id, n_targets, opt, &praw, false));
        delete praw;
        return HPDEX_OK;
    }

    // equal chunks of about nnz / kPipelineChunks entries (whole columns), uploaded in
    // descending order of their longest column: the compute left after the last copy is
    // about the last chunk's longest gene
    std::vector<long long> cb{0};
    for (int k = 1; k < kPipelineChunks; ++k) {
        const long long target = nnz / kPipelineChunks * k;
        const long long c = std::lower_bound(indptr, indptr + C + 1, target) - indptr;
        if (c > cb.back() && c < C) cb.push_back(c);
    }
    cb.push_back(C);
    const int K = (int)cb.size() - 1;
    std::vector<long long> longest((size_t)K, 0);
    long long max_chunk = 0;
    for (int k = 0; k < K; ++k) {
        max_chunk = std::max<long long>(max_chunk, (long long)(indptr[cb[k + 1]] - indptr[cb[k]]));
        for (long long c = cb[k]; c < cb[k + 1]; ++c)
            longest[(size_t)k] = std::max(longest[(size_t)k], m->col_nnz[(size_t)c]);
    }
    std::vector<int> seq((size_t)K);
    std::iota(seq.begin(), seq.end(), 0);
    std::stable_sort(seq.begin(), seq.end(), [&](int x, int y) { return longest[(size_t)x] > longest[(size_t)y]; });
    DevBuf<int32_t> queues;
    DevBuf<long long> stage[2];
    TRY(queues.alloc((size_t)K));
    // where the device reaches pageable host memory, a few CTAs read each chunk straight from the
    // caller's arrays (no staging, no driver copies); else cudaMemcpyAsync (int64 row ids through
    // staging buffers, narrowed on the device)
    const bool kernel_upload = m->dev.pageable_access;
    if (!idx32 && !kernel_upload)
        for (auto& b : stage) TRY(b.alloc((size_t)std::max<long long>(max_chunk, 1)));

    struct Res {  // copy stream, second compute stream and events of this call, released once
                  // their streams drained
        cudaStream_t copy = nullptr, comp2 = nullptr;
        std::vector<cudaEvent_t> ev;
        ~Res() {
            if (copy) cudaStreamSynchronize(copy);
            if (comp2) cudaStreamSynchronize(comp2);
            for (auto e : ev) if (e) cudaEventDestroy(e);
            if (copy) cudaStreamDestroy(copy);
            if (comp2) cudaStreamDestroy(comp2);
        }
    } r;
    // the copy stream at the highest priority: when SMs free up, a pending upload kernel's CTAs
    // take them before a rank kernel's
    int prio_least = 0, prio_greatest = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    CUDA_TRY(cudaStreamCreateWithPriority(&r.copy, cudaStreamNonBlocking, prio_greatest));
    CUDA_TRY(cudaStreamCreateWithFlags(&r.comp2, cudaStreamNonBlocking));
    r.ev.assign((size_t)(2 * K + 3), nullptr);
    for (auto& e : r.ev) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaStream_t sx = r.copy;
    auto enqueue_copy = [&](int j) -> int {  // upload position j: chunk seq[j], staging buffer j & 1
        const int k = seq[(size_t)j];
        const long long p0 = indptr[cb[k]], nk = indptr[cb[k + 1]] - p0;
        if (kernel_upload) {
            TRY(dispatch_dtype<UploadLaunch>(dtype, static_cast<const void*>(static_cast<const unsigned char*>(data) + p0 * vs),
                                             idx32 ? nullptr : indices + p0, idx32 ? indices32 + p0 : nullptr,
                                             static_cast<void*>(m->data.p + p0 * vs), m->rows.p + p0, nk,
                                             (long long)n_rows, sx));
            CUDA_TRY(cudaEventRecord(r.ev[2 * j], sx));
            return HPDEX_OK;
        }
        if (j >= 2 && !idx32) CUDA_TRY(cudaStreamWaitEvent(sx, r.ev[2 * (j - 2) + 1], 0));  // staging buffer free
        if (nk) {
            CUDA_TRY(cudaMemcpyAsync(m->data.p + p0 * vs, static_cast<const unsigned char*>(data) + p0 * vs,
                                     (size_t)nk * vs, cudaMemcpyHostToDevice, sx));
            if (idx32)
                CUDA_TRY(cudaMemcpyAsync(m->rows.p + p0, indices32 + p0, sizeof(int32_t) * nk, cudaMemcpyHostToDevice, sx));
            else
                CUDA_TRY(cudaMemcpyAsync(stage[j & 1].p, indices + p0, sizeof(int64_t) * nk, cudaMemcpyHostToDevice, sx));
        }
        CUDA_TRY(cudaEventRecord(r.ev[2 * j], sx));
        return HPDEX_OK;
    };

    // the host-side plan (group sizes, reference checks, layout, allocations) runs on a helper
    // thread while the first chunk is uploaded
    hpdex_plan* praw = nullptr;
    int plan_status = HPDEX_OK;
    std::string plan_error;
    const int dev_id = m->dev.device;
    std::thread planner([&] {
        cudaSetDevice(dev_id);
        plan_status = plan_create(m.get(), group_id, n_targets, opt, &praw, false);
        if (plan_status != HPDEX_OK) plan_error = hpdex_last_error();
    });
    // column pointers, then the first chunk; the per-chunk gene order while they upload
    int first_copy = HPDEX_OK;
    if (cudaMemcpyAsync(m->indptr.p, indptr, sizeof(int64_t) * ((size_t)C + 1), cudaMemcpyHostToDevice, sx) != cudaSuccess)
        first_copy = fail(HPDEX_ERR_CUDA, "column pointer upload failed");
    if (first_copy == HPDEX_OK) first_copy = enqueue_copy(0);
    std::vector<int32_t> order((size_t)C);  // each chunk's columns longest first
    for (int k = 0; k < K; ++k) {
        auto ob = order.begin() + cb[k], oe = order.begin() + cb[k + 1];
        std::iota(ob, oe, (int32_t)cb[k]);
        std::stable_sort(ob, oe, [&](int32_t x, int32_t y) { return m->col_nnz[(size_t)x] > m->col_nnz[(size_t)y]; });
    }
    planner.join();
    std::unique_ptr<hpdex_plan> p(praw);
    if (plan_status != HPDEX_OK) return fail(plan_status, "%s", plan_error.c_str());
    // the p-value kernel of each chunk writes U1 and P (straight into the caller's arrays
    // where the device can reach them), so the rank kernel keeps the tie sums
    p->fused_pvalues = false;
    p->ra.erfc_table = nullptr;
    TRY(first_copy);
    // Chunks alternate between two compute streams, so that the next chunk's rank kernel takes
    // the SMs of the previous one's last CTAs as they finish instead of waiting for all of them
    // (a chunk holds a few genes per CTA, so its tail is long). Chunks on the second stream use
    // a scratch set of their own.
    cudaStream_t sc2 = r.comp2;
    RankLayout lay2;
    TRY(rank_layout(m->dev, dtype, (int)p->G, m->max_col_nnz, &lay2, p->nbl, p->cnt_mode));
    DevBuf<unsigned char> dk2, dg2, ek2, eg2, acc2;
    DevBuf<uint32_t> cnt2;
    TRY(dk2.alloc(lay2.dk_bytes()));
    TRY(dg2.alloc(lay2.dg_bytes()));
    if (lay2.need_slab_scratch) {
        TRY(ek2.alloc(lay2.dk_bytes()));
        TRY(eg2.alloc(lay2.dg_bytes()));
    }
    if (!lay2.acc_in) TRY(acc2.alloc(lay2.acc_bytes((int)p->G)));
    TRY(cnt2.alloc(lay2.cnt_words((int)p->G)));
    const long long T = p->T;
    CUDA_TRY(cudaMemcpyAsync(p->order.p, order.data(), sizeof(int32_t) * C, cudaMemcpyHostToDevice, p->stream));

    // Output pages never written before (fresh numpy arrays) would fault one by one when the
    // device writes them; a host thread touches them while the first chunks are in flight, and
    // the compute stream waits for it before the first p-value kernel.
    // Page-locked outputs (hpdex_host_buffer_acquire) are written directly on any system and
    // need no touching; pageable ones directly where the device can reach pageable memory.
    bool pinned_out = false;
    if (U1_out && P_out) {
        cudaPointerAttributes a1{}, a2{};
        if (cudaPointerGetAttributes(&a1, U1_out) == cudaSuccess &&
            cudaPointerGetAttributes(&a2, P_out) == cudaSuccess)
            pinned_out = a1.type == cudaMemoryTypeHost && a2.type == cudaMemoryTypeHost;
        cudaGetLastError();
    }
    const bool direct = (m->dev.pageable_access || pinned_out) && U1_out && P_out;
    std::atomic<int> touched{pinned_out ? 1 : 0};
    struct Toucher {
        std::thread t;
        ~Toucher() { if (t.joinable()) t.join(); }
    } toucher;
    if (direct && !pinned_out) {
        const size_t bytes = sizeof(double) * (size_t)(T * C);
        toucher.t = std::thread([U1_out, P_out, bytes, &touched] {
            for (size_t o = 0; o < bytes; o += 4096) {
                reinterpret_cast<volatile unsigned char*>(U1_out)[o] = 0;
                reinterpret_cast<volatile unsigned char*>(P_out)[o] = 0;
            }
            touched.store(1, std::memory_order_release);
        });
    }
    cudaStream_t sc = p->stream;
    // every exit drains both compute streams before the plan, the toucher flag or the buffers go
    struct Drain {
        cudaStream_t s, s2;
        ~Drain() {
            cudaStreamSynchronize(s);
            cudaStreamSynchronize(s2);
        }
    } drain{sc, sc2};

    CUDA_TRY(cudaMemsetAsync(p->err.p, 0xff, kErrWords * sizeof(unsigned long long), sc));
    CUDA_TRY(cudaMemsetAsync(queues.p, 0, sizeof(int32_t) * K, sc));
    {
        const int grid = (int)std::max<long long>(1, std::min<long long>((n_rows + 255) / 256, (long long)m->dev.sms * 8));
        if (p->ra.acc_in_smem)
            prepare_group_ids_kernel<uint16_t><<<grid, 256, 0, sc>>>(p->gid.p, n_rows, (int32_t)p->G, reinterpret_cast<uint16_t*>(p->gidc.p));
        else
            prepare_group_ids_kernel<uint32_t><<<grid, 256, 0, sc>>>(p->gid.p, n_rows, (int32_t)p->G, reinterpret_cast<uint32_t*>(p->gidc.p));
        CUDA_TRY(cudaGetLastError());
    }
    cudaEvent_t ev_fork = r.ev[(size_t)(2 * K)], ev_join = r.ev[(size_t)(2 * K + 1)];
    cudaEvent_t ev_touch = r.ev[(size_t)(2 * K + 2)];
    CUDA_TRY(cudaEventRecord(ev_fork, sc));
    CUDA_TRY(cudaStreamWaitEvent(sc2, ev_fork, 0));
    for (int j = 0; j < K; ++j) {
        const int k = seq[(size_t)j];
        const long long c0 = cb[k], c1 = cb[k + 1];
        const long long p0 = indptr[c0], nk = indptr[c1] - p0;
        const bool second = kComputeStreams > 1 && (j & 1) != 0;
        cudaStream_t sj = second ? sc2 : sc;
        CUDA_TRY(cudaStreamWaitEvent(sj, r.ev[2 * j], 0));
        if (nk && !idx32 && !kernel_upload) {
            narrow_rows_kernel<<<(int)std::min<long long>((nk + 255) / 256, (long long)m->dev.sms * 16), 256, 0, sj>>>(
                stage[j & 1].p, m->rows.p + p0, nk, n_rows);
            CUDA_TRY(cudaGetLastError());
        }
        CUDA_TRY(cudaEventRecord(r.ev[2 * j + 1], sj));
        TRY(dispatch_dtype<KeyRangeLaunch>(dtype, (const void*)m->data.p, (const int64_t*)(m->indptr.p + c0), c1 - c0,
                                           m->col_kmin.p + c0, m->col_kmax.p + c0, m->col_has_zero.p + c0, nk,
                                           m->dev.sms, sj));
        RankArgs ra = p->ra;
        ra.order = p->order.p + c0;
        ra.n_order = (int32_t)(c1 - c0);
        ra.queue = queues.p + k;
        ra.single_gene = -1;
        if (second)
            set_layout_args(ra, lay2, (int)p->G, dk2.p, dg2.p, ek2.p, eg2.p, acc2.p, cnt2.p);
        // with kernel uploads, kUploadCTAs SMs stay free for the next chunk's upload (the last
        // chunk has none after it)
        const int grid = kernel_upload && j + 1 < K ? std::max(1, p->rank_grid - kUploadCTAs) : p->rank_grid;
        TRY(rank_status(rank_launch(dtype, ra, grid, p->rank_smem, sj), "rank kernel launch"));
        PArgs pa{};
        pa.U1 = p->U1.p;
        pa.P = p->P.p;
        pa.n = T * (c1 - c0);
        pa.n_cols = (int32_t)C;
        pa.col_lo = (int32_t)c0;
        pa.col_w = (int32_t)(c1 - c0);
        pa.U1_out = direct ? U1_out : nullptr;
        pa.P_out = direct ? P_out : nullptr;
        pa.group_rows = p->d_group_rows.p;
        pa.pk = p->d_pconst.p;
        pa.n1g = p->n1.p;
        pa.n2t = p->n2.p;
        pa.zero_handling = opt->zero_handling;
        pa.alternative = opt->alternative;
        pa.cc = opt->use_continuity ? 0.5 : 0.0;
        pa.fast = opt->fast_norm;
        if (direct && !pinned_out && j == 0) {
            CUDA_TRY(cudaLaunchHostFunc(sc, [](void* f) {
                const auto* done = static_cast<const std::atomic<int>*>(f);
                while (!done->load(std::memory_order_acquire)) std::this_thread::yield();
            }, &touched));
            CUDA_TRY(cudaEventRecord(ev_touch, sc));
        }
        if (direct && !pinned_out && j == 1)  // the second stream's p-values write those pages too
            CUDA_TRY(cudaStreamWaitEvent(sc2, ev_touch, 0));
        if (pa.n) {
            const int grid = (int)std::min<long long>((pa.n + 255) / 256, (long long)m->dev.sms * 8);
            mwu_pvalue_asymptotic_kernel<<<grid, 256, 0, sj>>>(pa);
            CUDA_TRY(cudaGetLastError());
        }
        if (j + 1 < K) TRY(enqueue_copy(j + 1));
    }
    CUDA_TRY(cudaEventRecord(ev_join, sc2));
    CUDA_TRY(cudaStreamWaitEvent(sc, ev_join, 0));
    CUDA_TRY(cudaStreamSynchronize(sc));
    TRY(check_device_errors(p.get()));
    if (!direct) TRY(hpdex_plan_download(p.get(), U1_out, P_out));
    return HPDEX_OK;
}

}  // namespace

// =======================================================================================
// Serving loop.
//
// A worker thread turns a stream of DE queries (a grouping over a resident matrix) into
// batched launches. Admission is in arrival order while the queries' device workspace fits the
// budget; the admitted queries of one value dtype (up to max_batch) become one launch of the
// persistent rank kernel with one task per query and one longest-first work queue of
// (query, gene) items, followed by one p-value kernel per query. Up to two batches are queued
// on the GPU at once, so the next batch is prepared while the previous one runs, and a query
// that arrives meanwhile joins the next launch. Completion is tracked per batch with an event;
// the worker then reads each query's error words, releases its workspace and wakes waiters.
// =======================================================================================
namespace {

// A batch stops growing once its queries hold this many matrix entries (about a millisecond
// of rank work on GB300): coalescing pays for small queries, whose launches would leave SMs
// idle, while a large query gains nothing from company and its neighbours would wait for it.
constexpr long long kServerBatchEntries = 48ll << 20;

struct ServerQuery {
    int64_t id = 0;
    int matrix = 0;
    long long T = 0, G = 0;
    hpdex_mwu_options opt{};
    std::vector<int32_t> gid;      // group ids (when no page-locked buffer was free)
    int32_t* gid_pinned = nullptr; // group ids in a page-locked pool buffer (asynchronous copy)
    std::vector<long long> group_rows;
    double* U1_out = nullptr;
    double* P_out = nullptr;
    size_t need = 0;  // device workspace bytes while admitted
    DevBuf<int32_t> d_gid;
    DevBuf<unsigned char> gidc;
    DevBuf<long long> d_group_rows;
    std::vector<PConst> pconst;  // per-target p-value constants (zero_handling min / max / mix)
    DevBuf<PConst> d_pconst;
    DevBuf<double> U1, P;
    DevBuf<uint32_t> n1, n2;
    DevBuf<unsigned long long> err;
    bool direct = false;  // p-values written straight into the host arrays
    int status = -1;      // -1 while pending or running
    std::string error;
    std::chrono::steady_clock::time_point t_submit, t_done;
    ~ServerQuery() {
        if (gid_pinned) host_pool().put(gid_pinned);
    }
};

struct ServerBatch {
    std::vector<ServerQuery*> q;
    DevBuf<RankTask> tasks;
    DevBuf<int32_t> order, queue;
    DevBuf<uint16_t> order_task;
    DevBuf<unsigned char> dk, dg, ek, eg, acc;
    DevBuf<uint32_t> cnt;
    DevBuf<PArgs> psets;       // the batch's p-value sets (one launch for all queries)
    DevBuf<long long> pfirst;
    // device time: t0 before the rank launch, tr after it, t1 after the p-values
    cudaEvent_t t0 = nullptr, tr = nullptr, t1 = nullptr;
    double prep_ms = 0.0;      // host time to prepare and queue the batch
    ~ServerBatch() {
        if (t0) cudaEventDestroy(t0);
        if (tr) cudaEventDestroy(tr);
        if (t1) cudaEventDestroy(t1);
    }
};

}  // namespace

struct hpdex_server {
    size_t budget = 0;
    int max_batch = 1;
    DeviceInfo dev;
    std::vector<hpdex_matrix*> mats;
    // per matrix: its genes in descending nnz, and the segment of that order holding each nnz
    // class floor(log2(nnz + 1)) = k: [seg[2k], seg[2k + 1]). A batch's work queue takes the
    // classes in descending order, each with every query's genes of that class: longest first
    // within a factor of two, built in time linear in the items (no sort per batch)
    std::vector<std::vector<int32_t>> mat_order;
    std::vector<std::vector<int64_t>> mat_class_start;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ServerQuery*> pending;
    std::map<int64_t, std::unique_ptr<ServerQuery>> queries;
    int64_t next_id = 1;
    size_t used = 0;
    bool stop = false;
    int64_t completed = 0, batches = 0;
    double busy_ms = 0.0;
    double rank_ms = 0.0, pvalue_ms = 0.0, prep_ms = 0.0;  // per phase, over all batches
    cudaStream_t stream = nullptr;
    std::thread worker;
};

namespace {

// Workspace of one admitted query: outputs, group ids (int32 and kernel type), group sizes,
// sample sizes under zero_handling=none.
size_t query_workspace(const hpdex_matrix* m, long long T, long long G, int zh) {
    const size_t tc = (size_t)(T * m->n_cols);
    size_t b = 16 * tc + 8 * (size_t)m->n_rows + 8 * (size_t)G + 64;
    if (zh == HPDEX_ZERO_NONE) b += 4 * tc + 4 * (size_t)m->n_cols;
    return b;
}

// Queues one batch on the server stream; on failure the caller fails its queries.
int server_launch(hpdex_server* S, ServerBatch& b) {
    cudaStream_t st = S->stream;
    const hpdex_matrix* m0 = S->mats[(size_t)b.q[0]->matrix];
    const int dtype = m0->dtype;
    int GL = 0;
    long long max_col = 0, items = 0;
    for (ServerQuery* q : b.q) {
        const hpdex_matrix* m = S->mats[(size_t)q->matrix];
        GL = std::max(GL, (int)q->G);
        max_col = std::max(max_col, m->max_col_nnz);
        items += m->n_cols;
    }
    RankLayout r;
    TRY(rank_layout(S->dev, dtype, GL, max_col, &r));
    TRY(b.dk.alloc(r.dk_bytes()));
    TRY(b.dg.alloc(r.dg_bytes()));
    if (r.need_slab_scratch) {
        TRY(b.ek.alloc(r.dk_bytes()));
        TRY(b.eg.alloc(r.dg_bytes()));
    }
    if (!r.acc_in) TRY(b.acc.alloc(r.acc_bytes(GL)));
    TRY(b.cnt.alloc(r.cnt_words(GL)));

    std::vector<RankTask> tasks(b.q.size());
    for (size_t i = 0; i < b.q.size(); ++i) {
        ServerQuery* q = b.q[i];
        const hpdex_matrix* m = S->mats[(size_t)q->matrix];
        const long long R = m->n_rows, C = m->n_cols, tc = q->T * C;
        TRY(q->d_gid.alloc((size_t)std::max<long long>(R, 1)));
        TRY(q->gidc.alloc((size_t)std::max<long long>(R, 1) * r.gb));
        TRY(q->d_group_rows.alloc((size_t)q->G));
        TRY(q->U1.alloc((size_t)std::max<long long>(tc, 1)));
        TRY(q->P.alloc((size_t)std::max<long long>(tc, 1)));
        if (q->opt.zero_handling == HPDEX_ZERO_NONE) {
            TRY(q->n1.alloc((size_t)std::max<long long>(C, 1)));
            TRY(q->n2.alloc((size_t)std::max<long long>(tc, 1)));
        }
        TRY(q->err.alloc(kErrWords));
        if (R) CUDA_TRY(cudaMemcpyAsync(q->d_gid.p, q->gid_pinned ? q->gid_pinned : q->gid.data(),
                                        sizeof(int32_t) * R, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(q->d_group_rows.p, q->group_rows.data(), sizeof(long long) * q->G, cudaMemcpyHostToDevice, st));
        q->pconst = target_consts(q->group_rows, q->opt.zero_handling);
        if (!q->pconst.empty()) {
            TRY(q->d_pconst.alloc(q->pconst.size()));
            CUDA_TRY(cudaMemcpyAsync(q->d_pconst.p, q->pconst.data(), sizeof(PConst) * q->pconst.size(), cudaMemcpyHostToDevice, st));
        }
        CUDA_TRY(cudaMemsetAsync(q->err.p, 0xff, kErrWords * sizeof(unsigned long long), st));
        const int grid = (int)std::max<long long>(1, std::min<long long>((R + 255) / 256, (long long)S->dev.sms * 8));
        if (r.acc_in)
            prepare_group_ids_kernel<uint16_t><<<grid, 256, 0, st>>>(q->d_gid.p, R, (int32_t)q->G, reinterpret_cast<uint16_t*>(q->gidc.p));
        else
            prepare_group_ids_kernel<uint32_t><<<grid, 256, 0, st>>>(q->d_gid.p, R, (int32_t)q->G, reinterpret_cast<uint32_t*>(q->gidc.p));
        CUDA_TRY(cudaGetLastError());
        RankTask& t = tasks[i];
        t.data = m->data.p;
        t.rows = m->rows.p;
        t.indptr = m->indptr.p;
        t.col_kmin = m->col_kmin.p;
        t.col_kmax = m->col_kmax.p;
        t.col_has_zero = m->col_has_zero.p;
        t.n_rows = R;
        t.n_cols = (int32_t)C;
        t.G = (int32_t)q->G;
        t.group_of_row = q->gidc.p;
        t.zero_handling = q->opt.zero_handling;
        t.tie_correction = q->opt.tie_correction;
        t.group_rows = q->d_group_rows.p;
        t.pconst = q->d_pconst.p;
        t.U1 = q->U1.p;
        t.tie = q->P.p;
        t.n1 = q->n1.p;
        t.n2 = q->n2.p;
        t.err = q->err.p;
        t.compact_decode = compact_decode(q->group_rows, R);
    }
    // one work queue over every (query, gene) item of the batch, longest first by nnz class
    std::vector<int32_t> order;
    std::vector<uint16_t> order_task;
    order.reserve((size_t)items);
    order_task.reserve((size_t)items);
    for (int k = 63; k >= 0; --k)
        for (size_t i = 0; i < b.q.size(); ++i) {
            const auto& ord = S->mat_order[(size_t)b.q[i]->matrix];
            const auto& seg = S->mat_class_start[(size_t)b.q[i]->matrix];
            const int64_t lo = seg[(size_t)(2 * k)], hi = seg[(size_t)(2 * k + 1)];
            order.insert(order.end(), ord.begin() + lo, ord.begin() + hi);
            order_task.insert(order_task.end(), (size_t)(hi - lo), (uint16_t)i);
        }
    TRY(b.tasks.alloc(tasks.size()));
    TRY(b.order.alloc(std::max<size_t>(order.size(), 1)));
    TRY(b.order_task.alloc(std::max<size_t>(order.size(), 1)));
    TRY(b.queue.alloc(1));
    CUDA_TRY(cudaMemcpyAsync(b.tasks.p, tasks.data(), sizeof(RankTask) * tasks.size(), cudaMemcpyHostToDevice, st));
    if (!order.empty()) {
        CUDA_TRY(cudaMemcpyAsync(b.order.p, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b.order_task.p, order_task.data(), sizeof(uint16_t) * order.size(), cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(cudaMemsetAsync(b.queue.p, 0, sizeof(int32_t), st));

    // results go straight into the caller's arrays when they are page-locked (result buffers
    // of hpdex_host_buffer_acquire) or when the device reaches pageable memory; pageable pages
    // that were never written would fault one by one when the device writes them: touch them
    for (ServerQuery* q : b.q) {
        bool pinned = false;
        cudaPointerAttributes a1{}, a2{};
        if (cudaPointerGetAttributes(&a1, q->U1_out) == cudaSuccess &&
            cudaPointerGetAttributes(&a2, q->P_out) == cudaSuccess)
            pinned = a1.type == cudaMemoryTypeHost && a2.type == cudaMemoryTypeHost;
        cudaGetLastError();
        q->direct = pinned || S->dev.pageable_access;
        if (!q->direct || pinned) continue;
        const size_t bytes = sizeof(double) * (size_t)(q->T * S->mats[(size_t)q->matrix]->n_cols);
        for (size_t o = 0; o < bytes; o += 4096) {
            reinterpret_cast<volatile unsigned char*>(q->U1_out)[o] = 0;
            reinterpret_cast<volatile unsigned char*>(q->P_out)[o] = 0;
        }
    }

    CUDA_TRY(cudaEventCreate(&b.t0));
    CUDA_TRY(cudaEventCreate(&b.tr));
    CUDA_TRY(cudaEventCreate(&b.t1));
    CUDA_TRY(cudaEventRecord(b.t0, st));
    if (!order.empty()) {
        RankArgs a{};
        a.tasks = b.tasks.p;
        a.order = b.order.p;
        a.order_task = b.order_task.p;
        a.n_order = (int32_t)order.size();
        a.queue = b.queue.p;
        a.single_gene = -1;
        bool any_int = false;  // the histogram variant when a query's matrix may hold integers
        for (auto* q : b.q) any_int = any_int || S->mats[(size_t)q->matrix]->has_int_cols;
        a.no_histogram = any_int ? 0 : 1;
        for (const RankTask& t : tasks) a.any_compact |= t.compact_decode;
        set_layout_args(a, r, GL, b.dk.p, b.dg.p, b.ek.p, b.eg.p, b.acc.p, b.cnt.p);
        TRY(rank_status(rank_launch(dtype, a, r.grid, r.smem, st), "rank kernel launch"));
    }
    CUDA_TRY(cudaEventRecord(b.tr, st));
    // the p-values of every query of the batch: one launch
    std::vector<PArgs> sets;
    std::vector<long long> first{0};
    for (ServerQuery* q : b.q) {
        const hpdex_matrix* m = S->mats[(size_t)q->matrix];
        PArgs pa{};
        pa.U1 = q->U1.p;
        pa.P = q->P.p;
        pa.n = q->T * m->n_cols;
        pa.n_cols = (int32_t)m->n_cols;
        pa.col_lo = 0;
        pa.col_w = (int32_t)m->n_cols;
        pa.U1_out = q->direct ? q->U1_out : nullptr;
        pa.P_out = q->direct ? q->P_out : nullptr;
        pa.group_rows = q->d_group_rows.p;
        pa.pk = q->d_pconst.p;
        pa.n1g = q->n1.p;
        pa.n2t = q->n2.p;
        pa.zero_handling = q->opt.zero_handling;
        pa.alternative = q->opt.alternative;
        pa.cc = q->opt.use_continuity ? 0.5 : 0.0;
        pa.fast = q->opt.fast_norm;
        sets.push_back(pa);
        first.push_back(first.back() + pa.n);
    }
    if (first.back() > 0) {
        TRY(b.psets.alloc(sets.size()));
        TRY(b.pfirst.alloc(first.size()));
        CUDA_TRY(cudaMemcpyAsync(b.psets.p, sets.data(), sizeof(PArgs) * sets.size(), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(b.pfirst.p, first.data(), sizeof(long long) * first.size(), cudaMemcpyHostToDevice, st));
        const int grid = (int)std::min<long long>((first.back() + 255) / 256, (long long)S->dev.sms * 8);
        mwu_pvalue_batch_kernel<<<grid, 256, 0, st>>>(b.psets.p, b.pfirst.p, (int)sets.size());
        CUDA_TRY(cudaGetLastError());
    }
    CUDA_TRY(cudaEventRecord(b.t1, st));
    return HPDEX_OK;
}

// Marks a query finished (caller holds S->mu) and releases its workspace.
void server_finish_query(hpdex_server* S, ServerQuery* q, int status, const std::string& msg) {
    if (q->gid_pinned) {  // its upload finished with the batch
        host_pool().put(q->gid_pinned);
        q->gid_pinned = nullptr;
    }
    q->status = status;
    q->error = msg;
    q->t_done = std::chrono::steady_clock::now();
    q->d_gid.alloc(0);
    q->gidc.alloc(0);
    q->d_group_rows.alloc(0);
    q->d_pconst.alloc(0);
    q->U1.alloc(0);
    q->P.alloc(0);
    q->n1.alloc(0);
    q->n2.alloc(0);
    q->err.alloc(0);
    S->used -= std::min(S->used, q->need);
    S->completed += 1;
}

// Results and errors of a finished batch.
void server_complete(hpdex_server* S, ServerBatch& b) {
    float ms = 0.0f, rms = 0.0f;
    cudaEventElapsedTime(&ms, b.t0, b.t1);
    cudaEventElapsedTime(&rms, b.t0, b.tr);
    std::vector<std::pair<int, std::string>> res;
    for (ServerQuery* q : b.q) {
        unsigned long long e[kErrWords];
        std::string msg;
        int st = HPDEX_OK;
        if (cudaMemcpy(e, q->err.p, sizeof e, cudaMemcpyDeviceToHost) != cudaSuccess) {
            st = HPDEX_ERR_CUDA;
            msg = "reading the error words failed";
        } else {
            st = decode_errors(e, q->G, &msg);
        }
        if (st == HPDEX_OK && !q->direct) {
            const size_t n = (size_t)(q->T * S->mats[(size_t)q->matrix]->n_cols);
            if (cudaMemcpy(q->U1_out, q->U1.p, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(q->P_out, q->P.p, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
                st = HPDEX_ERR_CUDA;
                msg = "copying the results failed";
            }
        }
        res.push_back({st, msg});
    }
    std::lock_guard<std::mutex> lock(S->mu);
    for (size_t i = 0; i < b.q.size(); ++i) server_finish_query(S, b.q[i], res[i].first, res[i].second);
    S->batches += 1;
    S->busy_ms += ms;
    S->rank_ms += rms;
    S->pvalue_ms += ms - rms;
    S->prep_ms += b.prep_ms;
    S->cv_done.notify_all();
}

void server_loop(hpdex_server* S) {
    cudaSetDevice(S->dev.device);
    std::deque<std::unique_ptr<ServerBatch>> inflight;
    for (;;) {
        // retire finished batches
        while (!inflight.empty()) {
            const cudaError_t e = cudaEventQuery(inflight.front()->t1);
            if (e == cudaErrorNotReady) break;
            cudaGetLastError();
            server_complete(S, *inflight.front());
            inflight.pop_front();
        }
        // admit the next batch while fewer than two are queued on the GPU
        std::unique_ptr<ServerBatch> b;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (inflight.empty() && S->pending.empty()) {
                if (S->stop) break;
                S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty(); });
                if (S->stop && S->pending.empty()) break;
            }
            if (inflight.size() < 2 && !S->pending.empty()) {
                b.reset(new ServerBatch());
                int dtype = -1;
                long long entries = 0;
                while (!S->pending.empty() && (int)b->q.size() < S->max_batch) {
                    ServerQuery* q = S->pending.front();
                    const int dt = S->mats[(size_t)q->matrix]->dtype;
                    if (dtype >= 0 && dt != dtype) break;
                    const long long e = S->mats[(size_t)q->matrix]->nnz;
                    if (!b->q.empty() && entries + e > kServerBatchEntries) break;
                    entries += e;
                    // a query larger than the whole budget runs alone on an idle server
                    const bool alone = b->q.empty() && inflight.empty() && S->used == 0;
                    if (S->used + q->need > S->budget && !alone) break;
                    S->pending.pop_front();
                    S->used += q->need;
                    dtype = dt;
                    b->q.push_back(q);
                }
                if (b->q.empty()) b.reset();
            }
            if (!b && !inflight.empty()) {
                // nothing to admit: wait for the oldest batch, or for a new arrival
                S->cv_work.wait_for(lk, std::chrono::microseconds(50));
                continue;
            }
        }
        if (!b) continue;
        const auto tp0 = std::chrono::steady_clock::now();
        const int lst = server_launch(S, *b);
        b->prep_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tp0).count();
        if (lst != HPDEX_OK) {
            const std::string msg = hpdex_last_error();
            cudaStreamSynchronize(S->stream);
            std::lock_guard<std::mutex> lock(S->mu);
            for (ServerQuery* q : b->q) server_finish_query(S, q, HPDEX_ERR_CUDA, msg);
            S->cv_done.notify_all();
            continue;
        }
        inflight.push_back(std::move(b));
    }
    for (auto& x : inflight) {
        cudaEventSynchronize(x->t1);
        server_complete(S, *x);
    }
}

}  // namespace

extern "C" {

int hpdex_server_create(int64_t workspace_bytes, int32_t max_batch, hpdex_server** out) {
    if (!out) return fail(HPDEX_ERR_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (workspace_bytes <= 0) return fail(HPDEX_ERR_ARGUMENT, "workspace_bytes must be positive");
    if (max_batch < 1 || max_batch > 65535) return fail(HPDEX_ERR_ARGUMENT, "max_batch must be in 1..65535");
    std::unique_ptr<hpdex_server> S(new hpdex_server());
    TRY(device_info(S->dev));
    TRY(ensure_erfc_table());
    S->budget = (size_t)workspace_bytes;
    S->max_batch = max_batch;
    CUDA_TRY(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    hpdex_server* raw = S.get();
    S->worker = std::thread([raw] { server_loop(raw); });
    *out = S.release();
    return HPDEX_OK;
}

int hpdex_server_add_matrix(hpdex_server* s, hpdex_matrix* m, int32_t* matrix_id) {
    if (!s || !m || !matrix_id) return fail(HPDEX_ERR_ARGUMENT, "NULL server, matrix or id pointer");
    if (m->dev.device != s->dev.device) return fail(HPDEX_ERR_ARGUMENT, "matrix and server are on different devices");
    std::vector<int32_t> order((size_t)m->n_cols);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return m->col_nnz[(size_t)a] > m->col_nnz[(size_t)b];
    });
    auto cls = [&](int32_t c) {
        const unsigned long long v = (unsigned long long)m->col_nnz[(size_t)c] + 1ull;
        return 63 - __builtin_clzll(v);
    };
    // classes fall along the descending order: class k is the segment [seg[2k], seg[2k + 1])
    std::vector<int64_t> seg(128, 0);
    for (size_t i = 0; i < order.size(); ++i) {
        const int k = cls(order[i]);
        if (seg[(size_t)(2 * k + 1)] == 0) seg[(size_t)(2 * k)] = (int64_t)i;
        seg[(size_t)(2 * k + 1)] = (int64_t)i + 1;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    s->mats.push_back(m);
    s->mat_order.push_back(std::move(order));
    s->mat_class_start.push_back(std::move(seg));
    *matrix_id = (int32_t)(s->mats.size() - 1);
    return HPDEX_OK;
}

int hpdex_server_submit(hpdex_server* s, int32_t matrix_id, const int32_t* group_id,
                        int64_t n_targets, const hpdex_mwu_options* opt, double* U1_out,
                        double* P_out, int64_t* query_id) {
    if (!s || !opt || !query_id || !U1_out || !P_out) return fail(HPDEX_ERR_ARGUMENT, "NULL argument");
    if (n_targets < 1) return fail(HPDEX_ERR_RUNTIME, "[mannwhitney] n_targets must be >= 1 (>=1 target groups)");
    if (n_targets >= (1ll << 30)) return fail(HPDEX_ERR_UNSUPPORTED, "n_targets too large");
    if (opt->method != HPDEX_ASYMPTOTIC) return fail(HPDEX_ERR_UNSUPPORTED, "the serving loop computes asymptotic p-values only");
    if (opt->zero_handling < 0 || opt->zero_handling > 3) return fail(HPDEX_ERR_ARGUMENT, "zero_handling must be 0..3");
    if (opt->alternative < 0 || opt->alternative > 2) return fail(HPDEX_ERR_ARGUMENT, "alternative must be 0..2");
    hpdex_matrix* m = nullptr;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (matrix_id < 0 || (size_t)matrix_id >= s->mats.size()) return fail(HPDEX_ERR_ARGUMENT, "unknown matrix id %d", matrix_id);
        m = s->mats[(size_t)matrix_id];
    }
    const long long R = m->n_rows, G = n_targets + 1;
    if (R > 0 && !group_id) return fail(HPDEX_ERR_ARGUMENT, "group_id is NULL");
    std::unique_ptr<ServerQuery> q(new ServerQuery());
    q->matrix = matrix_id;
    q->T = n_targets;
    q->G = G;
    q->opt = *opt;
    // a page-locked copy when the pool has one free: the worker's upload is then asynchronous
    q->gid_pinned = R > 0 ? static_cast<int32_t*>(host_pool().get(sizeof(int32_t) * (size_t)R)) : nullptr;
    if (q->gid_pinned) std::memcpy(q->gid_pinned, group_id, sizeof(int32_t) * (size_t)R);
    else q->gid.assign(group_id, group_id + R);
    q->group_rows.assign((size_t)G, 0);
    for (long long r = 0; r < R; ++r) {
        const int g = group_id[r];
        if (g >= 0 && g < G) ++q->group_rows[(size_t)g];
    }
    if (opt->zero_handling != HPDEX_ZERO_NONE && m->n_cols > 0) {  // as hpdex_plan_create
        if (q->group_rows[0] < 2) return fail(HPDEX_ERR_RUNTIME, "Sample too small for reference at column 0");
        for (long long g = 1; g < G; ++g)
            if (q->group_rows[(size_t)g] < 2) return fail(HPDEX_ERR_RUNTIME, "Sample too small for group %lld at column 0", g);
    }
    q->U1_out = U1_out;
    q->P_out = P_out;
    q->need = query_workspace(m, n_targets, G, opt->zero_handling);
    q->t_submit = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return fail(HPDEX_ERR_RUNTIME, "the server is shutting down");
    q->id = s->next_id++;
    *query_id = q->id;
    s->pending.push_back(q.get());
    s->queries[q->id] = std::move(q);
    s->cv_work.notify_one();
    return HPDEX_OK;
}

int hpdex_server_wait(hpdex_server* s, int64_t query_id, double timeout_s, double* latency_ms) {
    if (!s) return fail(HPDEX_ERR_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->queries.find(query_id);
    if (it == s->queries.end()) return fail(HPDEX_ERR_ARGUMENT, "unknown query id %lld", (long long)query_id);
    ServerQuery* q = it->second.get();
    auto done = [&] { return q->status >= 0; };
    if (timeout_s < 0) {
        s->cv_done.wait(lk, done);
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
        return fail(HPDEX_ERR_TIMEOUT, "query %lld still running after %.3f s", (long long)query_id, timeout_s);
    }
    if (latency_ms) latency_ms[0] = std::chrono::duration<double, std::milli>(q->t_done - q->t_submit).count();
    const int st = q->status;
    const std::string msg = q->error;
    s->queries.erase(it);
    if (st != HPDEX_OK) return fail(st, "%s", msg.c_str());
    return HPDEX_OK;
}

int hpdex_server_stats(const hpdex_server* s, int64_t* completed, int64_t* batches, double* busy_ms) {
    if (!s) return fail(HPDEX_ERR_ARGUMENT, "server is NULL");
    hpdex_server* w = const_cast<hpdex_server*>(s);
    std::lock_guard<std::mutex> lock(w->mu);
    if (completed) *completed = s->completed;
    if (batches) *batches = s->batches;
    if (busy_ms) *busy_ms = s->busy_ms;
    return HPDEX_OK;
}

int hpdex_server_phase_stats(const hpdex_server* s, double* prep_ms, double* rank_ms, double* pvalue_ms) {
    if (!s) return fail(HPDEX_ERR_ARGUMENT, "server is NULL");
    hpdex_server* w = const_cast<hpdex_server*>(s);
    std::lock_guard<std::mutex> lock(w->mu);
    if (prep_ms) *prep_ms = s->prep_ms;
    if (rank_ms) *rank_ms = s->rank_ms;
    if (pvalue_ms) *pvalue_ms = s->pvalue_ms;
    return HPDEX_OK;
}

int hpdex_server_destroy(hpdex_server* s) {
    if (!s) return HPDEX_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        while (!s->pending.empty()) {
            ServerQuery* q = s->pending.front();
            s->pending.pop_front();
            q->status = HPDEX_ERR_RUNTIME;
            q->error = "the server was destroyed before the query ran";
            q->t_done = std::chrono::steady_clock::now();
        }
        s->cv_work.notify_all();
        s->cv_done.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return HPDEX_OK;
}

}  // extern "C"

// =======================================================================================
// No-allocation entry point.
//
// For callers that must not allocate device memory during a call: code that runs inside a
// framework's own memory pool or caching allocator (where a cudaMalloc/cudaFree would
// bypass the pool and can synchronise the device), latency-critical serving paths that
// reserve all memory up front, and hosts embedding this library behind a plugin interface
// that forbids allocation. The caller passes device buffers for every input and output;
// the rest of the working memory is one file-scope device array of fixed size,
// kNoAllocScratchBytes, which every GPU that loads this library holds until process exit.
// =======================================================================================
namespace {

constexpr size_t kNoAllocScratchBytes = HPDEX_NOALLOC_SCRATCH_BYTES;  // 64 MiB per device
constexpr int kNoAllocMaxGroups = HPDEX_NOALLOC_MAX_GROUPS;           // n_targets + 1
constexpr long long kNoAllocMaxCols = HPDEX_NOALLOC_MAX_COLS;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
    unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
    DeviceInfo info;
};
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[64];

// Set-up, once per device, with that device current: the host-side symbol is only a
// stand-in, kernels must get the device address.
int noalloc_setup(int dev, NoAllocDevice** out) {
    if (dev < 0 || dev >= 64) return fail(HPDEX_ERR_UNSUPPORTED, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc_dev[dev];
    if (!d.scratch) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(HPDEX_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch) failed: %s",
                        cudaGetErrorString(e));
        TRY(device_info(d.info));
        TRY(ensure_erfc_table());
        d.scratch = static_cast<unsigned char*>(ptr);
    }
    *out = &d;
    return HPDEX_OK;
}

// group sizes (reference group_rows, mannwhitneyu.cpp:865-869), the longest column, and
// the identity gene order for the work queue
__global__ void noalloc_prepare_kernel(const int32_t* gid, long long n_rows, int G,
                                       const int64_t* indptr, int n_cols, long long* group_rows,
                                       unsigned long long* max_col, int32_t* order) {
    __shared__ unsigned int cnt[kNoAllocMaxGroups];
    for (int g = threadIdx.x; g < G; g += blockDim.x) cnt[g] = 0u;
    __syncthreads();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += stride) {
        const int g = gid[r];
        if (g >= 0 && g < G) atomicAdd(&cnt[g], 1u);
    }
    unsigned long long mx = 0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n_cols; c += stride) {
        const unsigned long long len = (unsigned long long)(indptr[c + 1] - indptr[c]);
        mx = len > mx ? len : mx;
        order[c] = (int32_t)c;
    }
    __syncthreads();
    for (int g = threadIdx.x; g < G; g += blockDim.x)
        if (cnt[g]) atomicAdd(reinterpret_cast<unsigned long long*>(&group_rows[g]), (unsigned long long)cnt[g]);
    mx = warp_max(mx);
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(max_col, mx);
}

}  // namespace

extern "C" int hpdex_mannwhitneyu_noalloc(int32_t dtype, const void* d_data, const int32_t* d_rows,
                                          const int64_t* d_indptr, int64_t n_rows, int64_t n_cols,
                                          const int32_t* d_group_id, int64_t n_targets,
                                          const hpdex_mwu_options* opt, double* d_U1,
                                          double* d_P, void* stream) {
    if (!opt) return fail(HPDEX_ERR_ARGUMENT, "options are NULL");
    if (n_targets < 1) return fail(HPDEX_ERR_RUNTIME, "[mannwhitney] n_targets must be >= 1 (>=1 target groups)");
    if (dtype_size(dtype) == 0) return fail(HPDEX_ERR_RUNTIME, "Unsupported dtype for data");
    if (opt->method != HPDEX_ASYMPTOTIC)
        return fail(HPDEX_ERR_UNSUPPORTED, "hpdex_mannwhitneyu_noalloc supports method=asymptotic only");
    if (opt->zero_handling < 0 || opt->zero_handling > 3) return fail(HPDEX_ERR_ARGUMENT, "zero_handling must be 0..3");
    if (opt->alternative < 0 || opt->alternative > 2) return fail(HPDEX_ERR_ARGUMENT, "alternative must be 0..2");
    if (n_targets + 1 > kNoAllocMaxGroups)
        return fail(HPDEX_ERR_UNSUPPORTED, "hpdex_mannwhitneyu_noalloc: n_targets + 1 = %lld exceeds %d",
                    (long long)(n_targets + 1), kNoAllocMaxGroups);
    if (n_cols < 0 || n_cols > kNoAllocMaxCols)
        return fail(HPDEX_ERR_UNSUPPORTED, "hpdex_mannwhitneyu_noalloc: n_cols = %lld outside [0, %lld]",
                    (long long)n_cols, kNoAllocMaxCols);
    if (n_rows < 0 || n_rows >= (1ll << 31)) return fail(HPDEX_ERR_UNSUPPORTED, "n_rows must be in [0, 2^31)");
    if (!d_indptr || (n_rows > 0 && !d_group_id) || (n_cols > 0 && n_targets > 0 && (!d_U1 || !d_P)))
        return fail(HPDEX_ERR_ARGUMENT, "NULL device pointer");
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    NoAllocDevice* nd = nullptr;
    TRY(noalloc_setup(dev, &nd));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int G = (int)(n_targets + 1);
    const long long C = n_cols, T = n_targets;
    const int zh = opt->zero_handling;
    const int kb = key_bytes(dtype);

    // carve the scratch: header | group_rows | per-column arrays | none-mode sizes | elements
    unsigned char* base = nd->scratch;
    size_t off = 0;
    auto take = [&](size_t bytes) { unsigned char* p = base + off; off = RankSmem::align16(off + bytes); return p; };
    int32_t* queue = reinterpret_cast<int32_t*>(take(sizeof(int32_t)));
    unsigned long long* err = reinterpret_cast<unsigned long long*>(take(kErrWords * sizeof(unsigned long long)));
    unsigned long long* max_col = reinterpret_cast<unsigned long long*>(take(sizeof(unsigned long long)));
    long long* group_rows = reinterpret_cast<long long*>(take(sizeof(long long) * G));
    RankTask* d_task = reinterpret_cast<RankTask*>(take(sizeof(RankTask)));
    const size_t header_bytes = off;
    int32_t* order = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * std::max<long long>(C, 1)));
    unsigned long long* kmin = reinterpret_cast<unsigned long long*>(take(8 * std::max<long long>(C, 1)));
    unsigned long long* kmax = reinterpret_cast<unsigned long long*>(take(8 * std::max<long long>(C, 1)));
    uint32_t* has_zero = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * std::max<long long>(C, 1)));
    uint32_t* n1 = nullptr;
    uint32_t* n2 = nullptr;
    if (zh == HPDEX_ZERO_NONE) {
        const size_t need = sizeof(uint32_t) * (size_t)(C + T * C);
        if (off + need > kNoAllocScratchBytes)
            return fail(HPDEX_ERR_UNSUPPORTED, "hpdex_mannwhitneyu_noalloc: zero_handling=none needs %zu scratch bytes for sample sizes", need);
        n1 = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * std::max<long long>(C, 1)));
        n2 = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * std::max<long long>(T * C, 1)));
    }

    // every call shares the array and finds the previous call's contents: clear what
    // must start at zero (work counter, group sizes, longest column) and reset the error words
    CUDA_TRY(cudaMemsetAsync(base, 0, header_bytes, s));
    CUDA_TRY(cudaMemsetAsync(err, 0xff, kErrWords * sizeof(unsigned long long), s));
    if (C == 0) {
        CUDA_TRY(cudaStreamSynchronize(s));
        return HPDEX_OK;
    }
    {
        const int grid = (int)std::min<long long>(std::max<long long>((std::max<long long>((long long)n_rows, C) + 255) / 256, 1),
                                                  (long long)nd->info.sms * 4);
        noalloc_prepare_kernel<<<grid, 256, 0, s>>>(d_group_id, n_rows, G, d_indptr, (int)C, group_rows,
                                                    max_col, order);
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) {
            cudaStreamSynchronize(s);
            return fail(HPDEX_ERR_CUDA, "no-alloc prepare kernel: %s", cudaGetErrorString(le));
        }
    }
    long long rows_host[kNoAllocMaxGroups];
    unsigned long long longest = 0;
    CUDA_TRY(cudaMemcpyAsync(rows_host, group_rows, sizeof(long long) * G, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(&longest, max_col, sizeof(longest), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    if (longest > 0 && (!d_data || !d_rows))
        return fail(HPDEX_ERR_ARGUMENT, "NULL device pointer (values or row ids of a matrix with entries)");
    if (zh != HPDEX_ZERO_NONE) {  // same checks and messages as hpdex_plan_create
        if (rows_host[0] < 2) return fail(HPDEX_ERR_RUNTIME, "Sample too small for reference at column 0");
        for (int g = 1; g < G; ++g)
            if (rows_host[g] < 2) return fail(HPDEX_ERR_RUNTIME, "Sample too small for group %d at column 0", g);
    }

    // rank-kernel layout (same sizing rule as the plan path); the accumulators must fit in
    // shared memory here, which kNoAllocMaxGroups guarantees
    const int nbl = 13;
    const size_t budget = std::min(nd->info.smem_per_sm - nd->info.smem_reserved, nd->info.smem_optin) - 2048;
    const int tie_warps = kRankThreads / 32;
    RankSmem L(nbl, G, tie_warps, 1, 1, 0, kb);
    if (L.total + 16384 > budget) return fail(HPDEX_ERR_UNSUPPORTED, "hpdex_mannwhitneyu_noalloc: layout does not fit");
    const int gb = group_bytes(1);
    int cap = (int)std::min<size_t>((budget - L.total) / (kb + gb + 1), (size_t)1 << 30);
    cap = std::max(0, cap - 8) & ~7;
    L = RankSmem(nbl, G, tie_warps, 1, 1, cap, kb);
    while (L.total > budget && cap > 0) {
        cap = std::max(0, cap - 64);
        L = RankSmem(nbl, G, tie_warps, 1, 1, cap, kb);
    }
    int blocks = 0;
    TRY(rank_status(rank_occupancy(dtype, L.total, nd->info.smem_optin, 1, &blocks), "rank kernel set-up"));
    if (blocks < 1) return fail(HPDEX_ERR_CUDA, "rank kernel does not fit on an SM");
    const int grid = nd->info.sms * blocks;
    // per CTA and warp: run counters (packed, and 32-bit for very large buckets)
    uint32_t* cnt_glob = reinterpret_cast<uint32_t*>(
        take(sizeof(uint32_t) * (size_t)grid * tie_warps * ((size_t)RankSmem::cnt_words(G) + G)));
    // group of each row, 16-bit
    uint16_t* gidc = reinterpret_cast<uint16_t*>(take((size_t)std::max<long long>(n_rows, 1) * gb));
    if (off > kNoAllocScratchBytes)
        return fail(HPDEX_ERR_UNSUPPORTED,
                    "hpdex_mannwhitneyu_noalloc: scratch exhausted: n_rows = %lld and n_targets = %lld "
                    "need %zu of the %zu bytes before any column slice", (long long)n_rows,
                    (long long)n_targets, off, kNoAllocScratchBytes);
    // per CTA: a decoded copy of the current column and, for columns larger than the
    // shared-memory capacity, a bucket-ordered slab slice
    const int nslices = (long long)longest > cap ? 2 : 1;
    off = (off + 127) & ~(size_t)127;  // slices in whole 128-byte lines
    const size_t left = off + 512 * (size_t)grid < kNoAllocScratchBytes ? kNoAllocScratchBytes - off - 512 * (size_t)grid : 0;
    const long long slice = (long long)(left / ((size_t)grid * nslices * (kb + gb))) & ~63ll;
    if (rank_slice((long long)longest) > slice)
        return fail(HPDEX_ERR_UNSUPPORTED,
                    "hpdex_mannwhitneyu_noalloc: a column holds %llu entries, above the %lld the "
                    "fixed scratch allows at this size", longest, slice);
    void* dk = take((size_t)grid * slice * kb);
    void* dg = take((size_t)grid * slice * gb);
    void* ek = nslices == 2 ? take((size_t)grid * slice * kb) : nullptr;
    void* eg = nslices == 2 ? take((size_t)grid * slice * gb) : nullptr;
    // from the first launch on, a failing step returns only after the stream has drained, so
    // that a failed call leaves no work of its own running on the shared array
    auto enqueue = [&]() -> int {
    {
        const int pg = (int)std::max<long long>(1, std::min<long long>((n_rows + 255) / 256, (long long)nd->info.sms * 8));
        prepare_group_ids_kernel<uint16_t><<<pg, 256, 0, s>>>(d_group_id, n_rows, G, gidc);
        CUDA_TRY(cudaGetLastError());
    }

    TRY(dispatch_dtype<KeyRangeLaunch>(dtype, d_data, d_indptr, C, kmin, kmax, has_zero, (long long)longest * C,
                                       nd->info.sms, s));
    RankTask t{};
    t.data = d_data;
    t.rows = d_rows;
    t.indptr = d_indptr;
    t.col_kmin = kmin;
    t.col_kmax = kmax;
    t.col_has_zero = has_zero;
    t.n_rows = n_rows;
    t.n_cols = (int32_t)C;
    t.G = G;
    t.group_of_row = gidc;
    t.zero_handling = zh;
    t.tie_correction = opt->tie_correction;
    t.group_rows = group_rows;
    t.U1 = d_U1;
    t.tie = d_P;
    t.n1 = n1;
    t.n2 = n2;
    t.err = err;
    CUDA_TRY(cudaMemcpyAsync(d_task, &t, sizeof(RankTask), cudaMemcpyHostToDevice, s));
    RankArgs a{};
    a.tasks = d_task;
    a.order = order;
    a.order_task = nullptr;
    a.n_order = (int32_t)C;
    a.queue = queue;
    a.single_gene = -1;
    a.G = G;
    a.dk_global = dk;
    a.dg_global = dg;
    a.ek_global = ek;
    a.eg_global = eg;
    a.slice = slice;
    a.acc_global = nullptr;
    a.cnt_global = cnt_glob;
    a.nb_max_log2 = nbl;
    a.elem_smem_cap = cap;
    a.acc_in_smem = 1;
    a.cnt_in_smem = 1;
    a.tie_warps = tie_warps;
    TRY(rank_status(rank_launch(dtype, a, grid, L.total, s), "rank kernel launch"));

    PArgs pa{};
    pa.U1 = d_U1;
    pa.P = d_P;
    pa.n = T * C;
    pa.n_cols = (int32_t)C;
    pa.col_lo = 0;
    pa.col_w = (int32_t)C;
    pa.group_rows = group_rows;
    pa.n1g = n1;
    pa.n2t = n2;
    pa.zero_handling = zh;
    pa.alternative = opt->alternative;
    pa.cc = opt->use_continuity ? 0.5 : 0.0;
    pa.fast = opt->fast_norm;
    mwu_pvalue_asymptotic_kernel<<<(int)std::min<long long>((pa.n + 255) / 256, (long long)nd->info.sms * 8), 256, 0, s>>>(pa);
    CUDA_TRY(cudaGetLastError());
    return HPDEX_OK;
    };
    if (const int rc = enqueue(); rc != HPDEX_OK) {
        cudaStreamSynchronize(s);
        return rc;
    }

    unsigned long long e[kErrWords];
    CUDA_TRY(cudaMemcpyAsync(e, err, sizeof e, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    const unsigned long long Gu = (unsigned long long)G;
    if (e[0] != ~0ull) {
        const unsigned long long c = e[0] / Gu, g = e[0] % Gu;
        if (g == 0) return fail(HPDEX_ERR_RUNTIME, "Sample too small for reference at column %llu", c);
        return fail(HPDEX_ERR_RUNTIME, "Sample too small for group %llu at column %llu", g, c);
    }
    if (e[1] != ~0ull) {
        const unsigned long long c = e[1] / Gu, g = e[1] % Gu;
        return fail(HPDEX_ERR_ARGUMENT, "column %llu stores more entries for group %llu than the group has rows "
                    "(duplicate row indices)", c, g);
    }
    return HPDEX_OK;
}
