// Batched transforms of uneven sizes: plan construction, work-queue layout,
// CUDA-graph capture and the C ABI (hpxfft_batch_*).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/hpxfft_gb300.h"
#include "batch.cuh"
#include "launch.cuh"

namespace hpxfft_gpu {

// plan.cu: records the calling thread's error message, returns status
int set_error(int status, const std::string &msg);
// plan.cu: the 2D plans' cached choices in wisdom files
void wisdom2d_write(FILE *f);
bool wisdom2d_check(const std::string &key, const std::vector<long long> &v);
void wisdom2d_add(const std::string &key, const std::vector<long long> &v);
void wisdom2d_forget();

namespace {

// dynamic shared memory limit of the batch kernel, once per device
template <class A>
cudaError_t prepare_batch_kernel()
{
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(batch_kernel<A>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

struct Tuning {
    int lag = 8;        // instances whose rows run ahead of their columns
    int ctas_per_sm = 2;
};

// Process-wide cache of tuned batch configurations, keyed by the multiset of
// shapes and the precision; exported to / imported from a text file.
std::mutex g_cache_mu;
std::map<std::string, Tuning> g_cache;

std::string cache_key(const std::vector<size_t> &nr, const std::vector<size_t> &nc, int prec)
{
    std::vector<std::pair<size_t, size_t>> v;
    for (size_t i = 0; i < nr.size(); ++i) v.push_back({nr[i], nc[i]});
    std::sort(v.begin(), v.end());
    std::string k = "p" + std::to_string(prec);
    size_t run = 0;
    for (size_t i = 0; i < v.size(); ++i) {
        ++run;
        if (i + 1 == v.size() || v[i + 1] != v[i]) {
            k += ";" + std::to_string(v[i].first) + "x" + std::to_string(v[i].second) + "*" + std::to_string(run);
            run = 0;
        }
    }
    return k;
}

}  // namespace
}  // namespace hpxfft_gpu

struct hpxfft_batch_s {
    int prec = HPXFFT_PREC_F32;
    size_t real_bytes = 4;
    std::vector<hpxfft_gpu::BatchInst> insts;
    std::vector<hpxfft_gpu::BatchDim> dims;
    std::vector<hpxfft_gpu::BatchItem> items;
    std::vector<size_t> offsets_bytes;
    size_t arena_bytes = 0;
    hpxfft_gpu::Tuning tune;
    // polls of a column item's bounded wait for its instance's rows
    long long spin_limit = 1ll << 24;
    // device tables
    hpxfft_gpu::BatchInst *d_insts = nullptr;
    hpxfft_gpu::BatchItem *d_items = nullptr;
    hpxfft_gpu::BatchDim *d_dims = nullptr;
    void *d_tw = nullptr;
    int *d_counters = nullptr;
    int *h_timeout = nullptr;  // pinned
    int grid = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    cudaEvent_t ev[2] = {};
    cudaEvent_t order[2] = {};  // caller stream -> own stream -> caller stream
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *graph_arena = nullptr;
    bool pending = false;
    std::map<std::string, double> meas;
};

namespace hpxfft_gpu {
namespace {

template <class A>
cudaError_t launch_batch(hpxfft_batch_s &b, void *arena, cudaStream_t st)
{
    BatchArgs a{};
    a.arena = arena;
    a.insts = b.d_insts;
    a.items = b.d_items;
    a.dims = b.d_dims;
    a.twpool = b.d_tw;
    a.nitems = (int)b.items.size();
    a.counters = b.d_counters;
    a.spin_limit = b.spin_limit;
    batch_kernel<A><<<b.grid, kBatchThreads, (size_t)padded_elems(b.prec == HPXFFT_PREC_F32 ? 8192 : 4096) * 2 *
                                                    b.real_bytes,
                      st>>>(a);
    return cudaGetLastError();
}

// queue order: rows of instance i, then columns of instance i - lag
void build_items(hpxfft_batch_s &b, const std::vector<int> &row_groups, const std::vector<int> &col_strips, int lag)
{
    b.items.clear();
    const int n = (int)b.insts.size();
    auto rows = [&](int i) {
        for (int g = 0; g < row_groups[i]; ++g) b.items.push_back({i, 0, g, 0});
    };
    auto cols = [&](int i) {
        for (int g = 0; g < col_strips[i]; ++g) b.items.push_back({i, 1, g, 0});
    };
    for (int i = 0; i < n + lag; ++i) {
        if (i < n) rows(i);
        if (i - lag >= 0) cols(i - lag);
    }
}

cudaError_t capture(hpxfft_batch_s &b, void *arena)
{
    if (b.exec) {
        cudaGraphExecDestroy(b.exec);
        b.exec = nullptr;
    }
    if (b.graph) {
        cudaGraphDestroy(b.graph);
        b.graph = nullptr;
    }
    // captured and replayed on the batch's own stream (the legacy default
    // stream cannot be captured); execute orders it against the caller's
    cudaStream_t st = b.own;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const size_t cbytes = sizeof(int) * (2 + b.insts.size());
    cudaError_t e1 = cudaMemsetAsync(b.d_counters, 0, cbytes, st);
    cudaError_t e2 = b.prec == HPXFFT_PREC_F32 ? launch_batch<ArithF32>(b, arena, st) : launch_batch<ArithFF>(b, arena, st);
    cudaError_t e3 = cudaMemcpyAsync(b.h_timeout, b.d_counters + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    e = cudaStreamEndCapture(st, &b.graph);
    if (e1 != cudaSuccess) return e1;
    if (e2 != cudaSuccess) return e2;
    if (e3 != cudaSuccess) return e3;
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(&b.exec, b.graph, 0);
    if (e != cudaSuccess) return e;
    b.graph_arena = arena;
    return cudaSuccess;
}

}  // namespace
}  // namespace hpxfft_gpu

using namespace hpxfft_gpu;

extern "C" {

int hpxfft_batch_create(hpxfft_batch *out, size_t count, const size_t *n_rows, const size_t *n_cols, int precision,
                        const char *plan_flag)
{
    if (!out) return set_error(HPXFFT_ERR_INVALID_ARG, "batch pointer is null");
    *out = nullptr;
    if (!hpxfft_plan_flag_valid(plan_flag)) return set_error(HPXFFT_ERR_INVALID_ARG, "Invalid FFTW plan flag string");
    if (precision != HPXFFT_PREC_F32 && precision != HPXFFT_PREC_F64)
        return set_error(HPXFFT_ERR_INVALID_ARG, "batches run in f32 or f64 (float-float)");
    if (count == 0 || !n_rows || !n_cols) return set_error(HPXFFT_ERR_INVALID_ARG, "empty batch");
    const auto t0 = std::chrono::steady_clock::now();
    hpxfft_batch_s *b = new (std::nothrow) hpxfft_batch_s();
    if (!b) return set_error(HPXFFT_ERR_ALLOC, "host allocation");
    b->prec = precision;
    b->real_bytes = precision == HPXFFT_PREC_F32 ? 4 : 8;
    // HPXFFT_BATCH_SPIN_LIMIT=n lowers the bound of the column items' wait
    // (n polls of 128 ns each), so a test can make it run out: the kernel
    // then skips the item and hpxfft_batch_synchronize reports
    // HPXFFT_ERR_TIMEOUT; the kernel returns either way
    if (const char *env = std::getenv("HPXFFT_BATCH_SPIN_LIMIT")) {
        char *end = nullptr;
        const long long v = std::strtoll(env, &end, 10);
        if (end != env && v >= 0) b->spin_limit = v;
    }
    const int maxel = precision == HPXFFT_PREC_F32 ? 8192 : 4096;
    const int cbytes = 2 * (int)b->real_bytes;
    std::map<std::tuple<int, int, int>, int> dim_index;  // (kind, L, log2W) -> dims
    std::map<int, int> tw_index;                         // table length -> pool offset
    int tw_total = 0;
    std::vector<int> row_groups, col_strips;
    size_t off = 0;
    auto fixed_id = [&](int kind, int L, int lw) -> int {
        if (precision != HPXFFT_PREC_F32) return -1;
#define HPXFFT_X(ID, L_, W_) \
    if (L == L_ && lw == W_) return ID;
        if (kind == 0) {
            HPXFFT_BATCH_ROWS_F32(HPXFFT_X)
        } else {
            HPXFFT_BATCH_COLS_F32(HPXFFT_X)
        }
#undef HPXFFT_X
        return -1;
    };
    auto dim_of = [&](int kind, int L, int lw) -> int {
        auto it = dim_index.find({kind, L, lw});
        if (it != dim_index.end()) return it->second;
        BatchDim d{};
        if (!factorize_radices(L, d.pp)) return -1;
        d.L = L;
        d.log2W = lw;
        d.fixed_id = fixed_id(kind, L, lw);
        d.ptab = 0;
        if (d.fixed_id >= 0) {
            // per-pass tables of the compile-time chain (same rule as FixedPasses)
            d.ptab = tw_total;
            for (int Ls = 1; Ls < L;) {
                const int R = fixed_radix(L, Ls, ArithF32::kEPTFixed);
                if (Ls > 1) tw_total += Ls * (R - 1);
                Ls *= R;
            }
        }
        b->dims.push_back(d);
        return dim_index[{kind, L, lw}] = (int)b->dims.size() - 1;
    };
    auto tw_of = [&](int len) {
        auto it = tw_index.find(len);
        if (it != tw_index.end()) return it->second;
        tw_index[len] = tw_total;
        tw_total += len;
        return tw_index[len];
    };
    for (size_t i = 0; i < count; ++i) {
        const size_t nx = n_rows[i], nc = n_cols[i];
        if (nx == 0 || nc < 4 || nc % 2 || nx > 65536 || nc > 65538) {
            delete b;
            return set_error(HPXFFT_ERR_UNSUPPORTED_SIZE, "instance " + std::to_string(i) + ": bad shape");
        }
        BatchInst in{};
        in.nx = (int)nx;
        in.dcy = (int)(nc / 2);
        in.M = in.dcy - 1;
        in.ncol = (int)nc;
        in.offset = (long long)(off / b->real_bytes);
        // rows: a whole row per CTA, short rows packed
        if (in.M > maxel || in.nx > maxel) {
            delete b;
            return set_error(HPXFFT_ERR_UNSUPPORTED_SIZE,
                             "instance " + std::to_string(i) + ": batched transforms hold one row and one column per CTA (at most " +
                                 std::to_string(maxel) + ")");
        }
        int rlw = 0;
        while (rlw < 6 && (in.M << (rlw + 1)) <= maxel && (1 << rlw) < in.nx) ++rlw;
        int clw = 6;
        while (clw > 0 && ((in.nx << clw) > maxel || (1 << (clw - 1)) >= in.dcy)) --clw;
        in.row_dim = dim_of(0, in.M, rlw);
        in.col_dim = dim_of(1, in.nx, clw);
        if (in.row_dim < 0 || in.col_dim < 0) {
            delete b;
            return set_error(HPXFFT_ERR_UNSUPPORTED_SIZE,
                             "instance " + std::to_string(i) + ": sizes must have no prime factor above 13");
        }
        in.tw_row = tw_of(2 * in.M);
        in.tw_col = tw_of(in.nx);
        in.row_items = (in.nx + (1 << rlw) - 1) >> rlw;
        row_groups.push_back(in.row_items);
        col_strips.push_back((in.dcy + (1 << clw) - 1) >> clw);
        b->insts.push_back(in);
        b->offsets_bytes.push_back(off);
        off += (nx * nc * b->real_bytes + 255) & ~(size_t)255;
    }
    b->arena_bytes = off;
    (void)cbytes;

    // tuned configuration from the cache, else the defaults
    const std::string key = cache_key(std::vector<size_t>(n_rows, n_rows + count),
                                      std::vector<size_t>(n_cols, n_cols + count), precision);
    bool cached = false;
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end()) {
            b->tune = it->second;
            cached = true;
        }
    }
    build_items(*b, row_groups, col_strips, b->tune.lag);

    cudaError_t e = precision == HPXFFT_PREC_F32 ? prepare_batch_kernel<ArithF32>() : prepare_batch_kernel<ArithFF>();
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
    b->stream = b->own;
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev[1]);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->order[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->order[1], cudaEventDisableTiming);
    const size_t twb = (size_t)tw_total * 2 * b->real_bytes;
    if (e == cudaSuccess) e = cudaMalloc(&b->d_insts, sizeof(BatchInst) * b->insts.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_items, sizeof(BatchItem) * b->items.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_dims, sizeof(BatchDim) * b->dims.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tw, twb);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, sizeof(int) * (2 + b->insts.size()));
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&b->h_timeout, sizeof(int), cudaHostAllocDefault);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_insts, b->insts.data(), sizeof(BatchInst) * b->insts.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_items, b->items.data(), sizeof(BatchItem) * b->items.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_dims, b->dims.data(), sizeof(BatchDim) * b->dims.size(), cudaMemcpyHostToDevice);
    for (auto &kv : tw_index) {
        if (e != cudaSuccess) break;
        char *dst = (char *)b->d_tw + (size_t)kv.second * 2 * b->real_bytes;
        e = precision == HPXFFT_PREC_F32 ? TwiddleLaunch<ArithF32>::full(dst, kv.first, b->stream)
                                         : TwiddleLaunch<ArithFF>::full(dst, kv.first, b->stream);
    }
    {
        // per-pass tables of every compile-time dim, at the offsets dim_of took
        for (auto &d : b->dims) {
            if (e != cudaSuccess || d.fixed_id < 0) continue;
            size_t off = (size_t)d.ptab;
            for (int Ls = 1; Ls < d.L;) {
                const int R = fixed_radix(d.L, Ls, ArithF32::kEPTFixed);
                if (Ls > 1) {
                    e = TwiddleLaunch<ArithF32>::pass((char *)b->d_tw + off * 2 * b->real_bytes, Ls, R, b->stream);
                    off += (size_t)Ls * (R - 1);
                }
                Ls *= R;
            }
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        hpxfft_batch_destroy(b);
        return set_error(HPXFFT_ERR_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
    }
    b->grid = sms * b->tune.ctas_per_sm;
    b->meas["plan"] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    b->meas["items"] = (double)b->items.size();
    b->meas["cached_plan"] = cached ? 1.0 : 0.0;
    double bytes = 0;
    for (auto &in : b->insts) bytes += 4.0 * (double)in.nx * in.dcy * 2.0 * (double)b->real_bytes;
    b->meas["algorithmic_bytes"] = bytes;

    // "measure" and stronger flags time a few queue lags and CTAs per SM on a
    // scratch arena and keep the fastest; the result is cached for this mix
    if (!cached && strcmp(plan_flag, "estimate") != 0) {
        void *arena = nullptr;
        if (cudaMalloc(&arena, b->arena_bytes) == cudaSuccess) {
            cudaMemsetAsync(arena, 0, b->arena_bytes, b->stream);
            Tuning best = b->tune;
            double best_ms = 1e30;
            const int lags[] = {0, 4, 8, 32};
            for (int lag : lags)
                for (int cps : {1, 2}) {
                    build_items(*b, row_groups, col_strips, lag);
                    cudaMemcpy(b->d_items, b->items.data(), sizeof(BatchItem) * b->items.size(), cudaMemcpyHostToDevice);
                    b->grid = sms * cps;
                    float ms = 0, sum = 0;
                    for (int rep = 0; rep < 3; ++rep) {
                        cudaMemsetAsync(b->d_counters, 0, sizeof(int) * (2 + b->insts.size()), b->stream);
                        cudaEventRecord(b->ev[0], b->stream);
                        cudaError_t le = precision == HPXFFT_PREC_F32 ? launch_batch<ArithF32>(*b, arena, b->stream)
                                                                       : launch_batch<ArithFF>(*b, arena, b->stream);
                        cudaEventRecord(b->ev[1], b->stream);
                        cudaEventSynchronize(b->ev[1]);
                        cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
                        if (le != cudaSuccess) ms = 1e9f;
                        if (rep) sum += ms;
                    }
                    if (sum < best_ms) {
                        best_ms = sum;
                        best.lag = lag;
                        best.ctas_per_sm = cps;
                    }
                }
            cudaFree(arena);
            b->tune = best;
            build_items(*b, row_groups, col_strips, best.lag);
            cudaMemcpy(b->d_items, b->items.data(), sizeof(BatchItem) * b->items.size(), cudaMemcpyHostToDevice);
            b->grid = sms * best.ctas_per_sm;
            b->meas["plan"] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            std::lock_guard<std::mutex> lock(g_cache_mu);
            g_cache[key] = best;
        } else {
            cudaGetLastError();
        }
    }
    b->meas["lag"] = b->tune.lag;
    b->meas["ctas_per_sm"] = b->tune.ctas_per_sm;
    *out = b;
    return HPXFFT_OK;
}

int hpxfft_batch_destroy(hpxfft_batch b)
{
    if (!b) return set_error(HPXFFT_ERR_STATE, "null batch");
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->d_insts);
    cudaFree(b->d_items);
    cudaFree(b->d_dims);
    cudaFree(b->d_tw);
    cudaFree(b->d_counters);
    if (b->h_timeout) cudaFreeHost(b->h_timeout);
    for (auto &ev : b->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : b->order)
        if (ev) cudaEventDestroy(ev);
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return HPXFFT_OK;
}

int hpxfft_batch_arena_bytes(hpxfft_batch b, size_t *bytes)
{
    if (!b || !bytes) return set_error(HPXFFT_ERR_INVALID_ARG, "null argument");
    *bytes = b->arena_bytes;
    return HPXFFT_OK;
}

int hpxfft_batch_offsets(hpxfft_batch b, size_t *offsets)
{
    if (!b || !offsets) return set_error(HPXFFT_ERR_INVALID_ARG, "null argument");
    std::copy(b->offsets_bytes.begin(), b->offsets_bytes.end(), offsets);
    return HPXFFT_OK;
}

int hpxfft_batch_set_stream(hpxfft_batch b, void *stream)
{
    if (!b) return set_error(HPXFFT_ERR_STATE, "null batch");
    b->stream = (cudaStream_t)stream;
    return HPXFFT_OK;
}

int hpxfft_batch_execute(hpxfft_batch b, void *d_arena)
{
    if (!b) return set_error(HPXFFT_ERR_STATE, "null batch");
    if (!d_arena || ((uintptr_t)d_arena & 255)) return set_error(HPXFFT_ERR_INVALID_ARG, "arena must be 256-byte aligned");
    if (b->pending) {
        int rc = hpxfft_batch_synchronize(b);
        if (rc != HPXFFT_OK) return rc;
    }
    cudaError_t e = cudaSuccess;
    if (!b->exec || b->graph_arena != d_arena) e = capture(*b, d_arena);
    if (e != cudaSuccess) return set_error(HPXFFT_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    const bool foreign = b->stream != b->own;
    if (foreign && ((e = cudaEventRecord(b->order[0], b->stream)) != cudaSuccess ||
                    (e = cudaStreamWaitEvent(b->own, b->order[0], 0)) != cudaSuccess))
        return set_error(HPXFFT_ERR_CUDA, std::string("stream order: ") + cudaGetErrorString(e));
    if ((e = cudaEventRecord(b->ev[0], b->own)) != cudaSuccess || (e = cudaGraphLaunch(b->exec, b->own)) != cudaSuccess ||
        (e = cudaEventRecord(b->ev[1], b->own)) != cudaSuccess)
        return set_error(HPXFFT_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    if (foreign && ((e = cudaEventRecord(b->order[1], b->own)) != cudaSuccess ||
                    (e = cudaStreamWaitEvent(b->stream, b->order[1], 0)) != cudaSuccess))
        return set_error(HPXFFT_ERR_CUDA, std::string("stream order: ") + cudaGetErrorString(e));
    b->pending = true;
    return HPXFFT_OK;
}

int hpxfft_batch_synchronize(hpxfft_batch b)
{
    if (!b) return set_error(HPXFFT_ERR_STATE, "null batch");
    if (!b->pending) return HPXFFT_OK;
    cudaError_t e = cudaEventSynchronize(b->ev[1]);
    b->pending = false;
    if (e != cudaSuccess) return set_error(HPXFFT_ERR_CUDA, std::string("batch: ") + cudaGetErrorString(e));
    float ms = 0;
    cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
    b->meas["total"] = 1e-3 * ms;
    if (*b->h_timeout) return set_error(HPXFFT_ERR_TIMEOUT, "a column item gave up waiting for its rows");
    return HPXFFT_OK;
}

int hpxfft_batch_get_measurement(hpxfft_batch b, const char *name, double *value)
{
    if (!b || !name || !value) return set_error(HPXFFT_ERR_INVALID_ARG, "null argument");
    int rc = hpxfft_batch_synchronize(b);
    if (rc != HPXFFT_OK) return rc;
    auto it = b->meas.find(name);
    *value = it == b->meas.end() ? 0.0 : it->second;
    return HPXFFT_OK;
}

int hpxfft_wisdom_export(const char *path)
{
    if (!path) return set_error(HPXFFT_ERR_INVALID_ARG, "null path");
    FILE *f = fopen(path, "w");
    if (!f) return set_error(HPXFFT_ERR_IO, std::string("Failed to open file: ") + path);
    fprintf(f, "hpxfft-gb300-wisdom 2\n");
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        for (auto &kv : g_cache) fprintf(f, "%s %d %d\n", kv.first.c_str(), kv.second.lag, kv.second.ctas_per_sm);
    }
    wisdom2d_write(f);
    fclose(f);
    return HPXFFT_OK;
}

// Version 1 files hold batch entries ("key lag ctas_per_sm"); version 2 adds
// 2D plan entries ("2d;... columns ff_pairs tc_vectors tc_rows").  A file
// with any malformed entry is rejected whole: nothing of it is merged.
int hpxfft_wisdom_import(const char *path)
{
    if (!path) return set_error(HPXFFT_ERR_INVALID_ARG, "null path");
    FILE *f = fopen(path, "r");
    if (!f) return set_error(HPXFFT_ERR_IO, std::string("Failed to open file: ") + path);
    std::vector<std::string> lines;
    {
        std::string cur;
        int ch;
        while ((ch = fgetc(f)) != EOF) {
            if (ch == '\n') {
                lines.push_back(cur);
                cur.clear();
            } else {
                cur.push_back((char)ch);
            }
        }
        if (!cur.empty()) lines.push_back(cur);
    }
    fclose(f);
    int version = 0;
    {
        char head[64] = {};
        if (lines.empty() || sscanf(lines[0].c_str(), "%63s %d", head, &version) != 2 ||
            strcmp(head, "hpxfft-gb300-wisdom") || (version != 1 && version != 2))
            return set_error(HPXFFT_ERR_INVALID_ARG, "not a wisdom file");
    }
    std::vector<std::pair<std::string, Tuning>> rows;
    std::vector<std::pair<std::string, std::vector<long long>>> rows2d;
    for (size_t i = 1; i < lines.size(); ++i) {
        const std::string &ln = lines[i];
        if (ln.find_first_not_of(" \t\r") == std::string::npos) continue;
        const size_t sp = ln.find(' ');
        if (sp == std::string::npos || sp == 0) return set_error(HPXFFT_ERR_INVALID_ARG, "corrupt wisdom entry");
        const std::string key = ln.substr(0, sp);
        std::vector<long long> v;
        const char *q = ln.c_str() + sp;
        for (;;) {
            while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
            if (!*q) break;
            char *end = nullptr;
            const long long x = strtoll(q, &end, 10);
            if (end == q) return set_error(HPXFFT_ERR_INVALID_ARG, "corrupt wisdom entry");
            v.push_back(x);
            q = end;
        }
        if (key.rfind("2d;", 0) == 0) {
            if (version < 2 || !wisdom2d_check(key, v)) return set_error(HPXFFT_ERR_INVALID_ARG, "corrupt wisdom entry");
            rows2d.push_back({key, v});
            continue;
        }
        if (v.size() != 2 || v[0] < 0 || v[0] > 4096 || v[1] < 1 || v[1] > 8)
            return set_error(HPXFFT_ERR_INVALID_ARG, "corrupt wisdom entry");
        Tuning t;
        t.lag = (int)v[0];
        t.ctas_per_sm = (int)v[1];
        rows.push_back({key, t});
    }
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        for (auto &r : rows) g_cache[r.first] = r.second;
    }
    for (auto &r : rows2d) wisdom2d_add(r.first, r.second);
    return HPXFFT_OK;
}

int hpxfft_wisdom_forget(void)
{
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        g_cache.clear();
    }
    wisdom2d_forget();
    return HPXFFT_OK;
}

}  // extern "C"
