// Plan construction and the C ABI (include/hpxfft_gb300.h).
//
// A plan mirrors what hpxfft::shared::loop::initialize builds
// (core/src/shared/loop.cpp:158-189): the dimensions derived from the padded
// buffer (dim_c_x = n_row, dim_c_y = n_col/2, dim_r_y = 2*dim_c_y - 2), one
// row plan and one column plan.  Instead of FFTW plans it holds the launch
// shapes of the row kernel and of the one or two column kernels, their radix
// sequences and FP64-generated twiddle tables in HBM.  Also here: the
// split-BF16 tensor-core stages, the host-buffer entry points (zero-copy on
// page-locked memory), the 3D plans and the allocation-free entry point.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>
#include <string>

#include "../../include/hpxfft_gb300.h"
#include "bluestein.cuh"
#include "launch.cuh"

namespace hpxfft_gpu {

static thread_local std::string g_last_error;
constexpr int kMaxDevices = 64;
// what a plan transforms: both passes, the column pass alone, the row pass alone
constexpr int kPlanFull = 0, kPlanColumns = 1, kPlanRows = 2;

static int fail(int status, const std::string &msg)
{
    g_last_error = msg;
    return status;
}
int set_error(int status, const std::string &msg) { return fail(status, msg); }

static int cuda_fail(cudaError_t e, const char *what)
{
    return fail(HPXFFT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// The plan's tunable choices; -1 leaves a choice to the fixed rules.
//   columns     1: single-kernel (cluster) column pass, 2: two-kernel four-step pass
//   ff_pairs    float-float forward: raw (hi, lo) pairs between the kernels (1) or doubles (0)
//   tc_vectors  split-BF16 column steps: 256 or 512 length-16 vectors per CTA
//   tc_rows     split-BF16: tensor-core rows (1) or FP32 rows (0)
struct PlanChoice {
    int columns = -1;
    int ff_pairs = -1;
    int tc_vectors = -1;
    int tc_rows = -1;
};

struct DimPlan {
    LaunchShape shape{};
    PassPlan pp{};
    int C = 1;
    int log2W = 0;
    int L = 0;
    int FL = 0;              // L when a compile-time pass chain is used, else 0
    void *ptab = nullptr;    // per-pass twiddles of that chain
};

// A dimension the direct kernels do not cover, run through a columns-only
// plan `sub` of length M on a scratch array of `width` complex columns:
// Bluestein's convolution (M the power of two >= 2L - 1) or, for rows
// longer than a cluster holds, the length-L transform itself (M = L) on a
// transposed copy.
struct AltAxis {
    bool on = false;
    bool bluestein = false;
    size_t L = 0, M = 0;
    size_t width = 0;
    hpxfft_plan sub = nullptr;
    // tables in the plan's arithmetic (alt_mode: float-float pairs for the
    // FP64 plan, the column steps' compute type)
    void *chirp = nullptr;   // L entries exp(-i pi n^2 / L)
    void *kernel = nullptr;  // M entries: DFT_M of the conjugate chirp, over M
    void *wtab = nullptr;    // rows: W_2L^k, k = 0..L
    // the column steps apply chirp and kernel while loading and storing
    // (the sub-plan takes the two-kernel pass)
    bool fused = false;
    // float-float plans: steps A and B of the sub-plan exchange raw pairs
    // with one exponent per step-A block (as the FP64 plan's own steps do)
    int *exp_blocks = nullptr;
};

}  // namespace hpxfft_gpu

struct hpxfft_plan_s {
    size_t nx = 0, ny = 0, M = 0, dcy = 0, ncol = 0, batch = 1;
    int prec = HPXFFT_PREC_F64;
    std::string flag;
    size_t real_bytes = 8;  // bytes of one storage real
    size_t tw_elem = 16;    // bytes of one complex twiddle
    hpxfft_gpu::DimPlan row, col;
    // two-kernel column pass (nx = N1 * N2): step A then step B through scratch
    bool col_two_step = false;
    int N1 = 0, N2 = 0;
    hpxfft_gpu::DimPlan colA, colB;
    void *scratch = nullptr;
    // float-float forward two-step pass: rows -> step A -> step B exchange
    // raw (hi, lo) pairs with per-row / per-block exponents instead of doubles
    bool ff_pairs = false;
    // float-float forward column steps with warp-local passes
    // (HPXFFT_FF_WARP_COLS=0 keeps the CTA-wide passes: tests, tuning)
    bool ff_warp_cols = true;
    // float-float forward rows of 8192 pairs with radix-16 passes
    // (RowLaunchFF16): their own pass tables and launch shape; the c2r keeps
    // the radix-8 chain of `row`
    bool ff_row16 = false;
    void *row16_ptab = nullptr;
    hpxfft_gpu::LaunchShape row16_shape{};
    // float-float rows of 16384 pairs as two kernels instead of a two-CTA
    // cluster: the DFTs of the rows' halves (radix-16 chain, into the column
    // scratch or half_buf), then the radix-2 combination and the split
    bool row_halves = false;
    int *half_exp = nullptr;              // [batch][2 nx] exponents of the half-rows
    void *half_buf = nullptr;             // when the plan has no column scratch
    void *half_wz = nullptr, *half_ws = nullptr;  // W_M^k, W_2M^k, k <= M/2
    int *exp_rows = nullptr;   // [batch][nx]
    int *exp_step_a = nullptr; // [batch][step A blocks]
    // split-BF16 precision: both column steps (and the rows, for compiled
    // row shapes) on the tensor cores
    bool tc_cols = false;
    bool tc_rows = false;
    void *tc_dft = nullptr;     // BF16 DFT-16 matrix splits
    int *dev_error = nullptr;   // set by a tensor-core kernel whose wait gave up
    void *tw_row = nullptr, *tw_col = nullptr;
    void *dbuf = nullptr;
    size_t dbuf_bytes = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    // kernel timing ring: slot i holds events before the first kernel, between
    // the two kernels and after the second; slots [done, next) are unread
    static constexpr int kSlots = 64;
    cudaEvent_t kev[kSlots][4] = {};  // [3]: between column steps A and B
    long long next = 0, done = 0;
    cudaEvent_t ev_copy[2] = {};  // before the host->device copy, after the device->host copy
    bool pending_copy = false;
    bool last_zero_copy = false;  // the last host-buffer transform read and wrote host memory directly
    // chunked host transfers overlapped with the kernels (two-step plans):
    // copy streams and per-chunk events, made on first use
    static constexpr int kChunks = 8;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t chunk_in[kChunks] = {}, chunk_b[kChunks] = {}, chunk_out[kChunks] = {};
    bool last_pipelined = false;  // the last host-buffer transform took that path
    bool columns_only = false;    // the column pass alone (the first axis of a 3D transform)
    bool rows_only = false;       // the row pass alone (the local rows of a slab decomposition)
    double peak_gbps = 0.0;       // nominal DRAM bandwidth of the device (memory clock x bus width)
    double sum_first = 0, sum_second = 0, sum_total = 0, sum_step_a = 0;
    long long nsum = 0;
    std::map<std::string, double> meas;
    hpxfft_gpu::PlanChoice choice;  // the choices in effect (resolved, no -1)
    // plan search under "measure" and stronger flags: each distinct candidate
    // and its best time (ms); empty for "estimate" and for a cached choice
    std::vector<std::pair<std::string, double>> tuning;
    std::string tuned_from;  // "rules", "search" or "wisdom"
    // rows / columns outside the direct kernels' sizes, and their scratch
    // array (the two run one after the other on the plan's stream)
    hpxfft_gpu::AltAxis alt_row, alt_col;
    void *alt_buf = nullptr;
};

namespace hpxfft_gpu {

// Elements of one CTA's transform(s): 4096 float-float (or FP64) pairs or
// 8192 FP32 pairs, 64 KB of data, so two CTAs share an SM.
// FP32 storage: the FP32 path and the split-BF16 path (FP32 outside the
// tensor-core stage)
static bool f32_storage(int prec) { return prec == HPXFFT_PREC_F32 || prec == HPXFFT_PREC_BF16X3; }

static int max_elems_for(int prec) { return f32_storage(prec) ? 8192 : 4096; }

// arithmetic of the Bluestein / transposing kernels and format of their
// tables: FP32, float-float on FP64 storage (the FP64 plan), DFMA FP64
static int alt_mode(int prec)
{
    return f32_storage(prec) ? kTabF32 : prec == HPXFFT_PREC_F64 ? kTabFF : kTabF64;
}

static int threads_for(int nel)
{
    int t = (nel + kElemsPerThread - 1) / kElemsPerThread;
    t = (t + 31) / 32 * 32;
    return t < 32 ? 32 : t;
}

// Rows: the smallest cluster whose CTAs hold a row each; short rows are
// packed (up to 16 per CTA) to fill the CTA.
static bool plan_rows(hpxfft_plan_s &p)
{
    // float-float rows of 8192 pairs fit one 1024-thread CTA: faster than a
    // 2-CTA cluster split (measured on 16384^2: 4.3 vs 5.1 ms); shorter rows
    // are packed only up to the compiled 4096-pair shapes
    const int maxel = p.prec == HPXFFT_PREC_F64 ? 8192 : max_elems_for(p.prec);
    const int packel = max_elems_for(p.prec);
    const size_t cbytes = 2 * p.real_bytes;
    for (int C : {1, 2, 4}) {
        if (p.M % C) continue;
        const int L = (int)(p.M / C);
        if (C > 1 && L % C) continue;
        if (L > maxel) continue;
        PassPlan pp;
        if (!factorize_radices(L, pp)) return false;
        int log2W = 0;
        if (C == 1)
            while (log2W < 4 && (L << (log2W + 1)) <= packel && ((size_t)1 << log2W) < p.nx) ++log2W;
        DimPlan &d = p.row;
        d.C = C;
        d.L = L;
        d.log2W = log2W;
        d.pp = pp;
        const int nel = L << log2W;
        d.shape.threads = threads_for(nel);
        d.shape.smem = (size_t)padded_elems(nel) * cbytes;
        d.shape.cluster = C;
        const size_t groups = (p.nx + ((size_t)1 << log2W) - 1) >> log2W;
        d.shape.grid = dim3((unsigned)(groups * C), (unsigned)p.batch, 1);
        return true;
    }
    return false;
}

// Columns: strips as wide as possible (64-byte row segments: 4 float-float
// or 8 FP32 columns), then the smallest cluster that holds the strip.
static bool plan_cols(hpxfft_plan_s &p)
{
    const int maxel = max_elems_for(p.prec);
    const size_t cbytes = 2 * p.real_bytes;
    int pref = f32_storage(p.prec) ? 3 : 2;
    while (pref > 0 && ((size_t)1 << (pref - 1)) >= p.dcy) --pref;
    for (int log2W = pref; log2W >= 0; --log2W) {
        for (int C : {1, 2, 4, 8, 16}) {
            if (p.nx % C) continue;
            const int L = (int)(p.nx / C);
            if (C > 1 && L % C) continue;
            if ((L << log2W) > maxel) continue;
            PassPlan pp;
            if (!factorize_radices(L, pp)) return false;
            DimPlan &d = p.col;
            d.C = C;
            d.L = L;
            d.log2W = log2W;
            d.pp = pp;
            const int nel = L << log2W;
            d.shape.threads = threads_for(nel);
            d.shape.smem = (size_t)padded_elems(nel) * cbytes;
            d.shape.cluster = C;
            const size_t strips = (p.dcy + ((size_t)1 << log2W) - 1) >> log2W;
            d.shape.grid = dim3((unsigned)(strips * C), (unsigned)p.batch, 1);
            return true;
        }
    }
    return false;
}

static bool has_fixed_step(int prec, const DimPlan &d)
{
    switch (prec) {
    case HPXFFT_PREC_F64: return ColStepLaunch<ArithFF>::has_fixed(d.L, d.log2W);
    case HPXFFT_PREC_F32: return ColStepLaunch<ArithF32>::has_fixed(d.L, d.log2W);
    case HPXFFT_PREC_BF16X3: return TcColStepLaunch::supports(d.L);  // FP32 chain after the tensor-core pass
    default: return false;
    }
}

// Shapes of the two-kernel column pass for power-of-two nx >= 1024:
// N2 = 2^floor(log2(nx)/2) (step A length), N1 = nx / N2 (step B length),
// strips of up to 64 columns.
static bool plan_colsteps(hpxfft_plan_s &p)
{
    if (p.nx < 1024 || (p.nx & (p.nx - 1))) return false;
    int lg = 0;
    while (((size_t)1 << lg) < p.nx) ++lg;
    p.N2 = 1 << (lg / 2);
    p.N1 = (int)(p.nx / p.N2);
    const int maxel = max_elems_for(p.prec);
    const size_t cbytes = 2 * p.real_bytes;
    if (p.prec == HPXFFT_PREC_BF16X3) {
        // tensor-core steps: nv length-16 vectors per CTA, 16 nv / L columns;
        // 256 (four CTAs per SM) measured faster than 512 on 16384^2 (1.91 vs
        // 2.18 ms) and is the rule; the plan's choice may set 512
        const int nv = p.choice.tc_vectors == 512 ? 512 : 256;
        for (int step = 0; step < 2; ++step) {
            DimPlan &d = step == 0 ? p.colA : p.colB;
            const int L = step == 0 ? p.N2 : p.N1;
            if (!TcColStepLaunch::supports(L) || !factorize_radices(L, d.pp)) return false;
            d.C = 1;
            d.L = L;
            d.log2W = TcColStepLaunch::log2W(L, nv);
            d.shape.threads = TcColStepLaunch::threads(nv);
            d.shape.smem = TcColStepLaunch::smem(nv);
            d.shape.cluster = 1;
            const size_t strips = (p.dcy + ((size_t)1 << d.log2W) - 1) >> d.log2W;
            const size_t groups = step == 0 ? (size_t)p.N1 : (size_t)p.N2;
            d.shape.grid = dim3((unsigned)(groups * strips), (unsigned)p.batch, 1);
        }
        return true;
    }
    int wcap = 6;  // at most 64 columns per strip
    while (wcap > 0 && ((size_t)1 << (wcap - 1)) >= p.dcy) --wcap;
    for (int step = 0; step < 2; ++step) {
        DimPlan &d = step == 0 ? p.colA : p.colB;
        const int L = step == 0 ? p.N2 : p.N1;
        int log2W = wcap;
        while (log2W > 0 && (L << log2W) > maxel) --log2W;
        if ((L << log2W) > maxel) return false;
        // narrow arrays keep the compiled strip width (idle columns are
        // masked) rather than fall back to the runtime-plan kernel
        int full = 6;
        while (full > 0 && (L << full) > maxel) --full;
        d.L = L;
        d.log2W = full;
        if (full > log2W && has_fixed_step(p.prec, d)) log2W = full;
        PassPlan pp;
        if (!factorize_radices(L, pp)) return false;
        d.C = 1;
        d.L = L;
        d.log2W = log2W;
        d.pp = pp;
        const int nel = L << log2W;
        d.shape.threads = threads_for(nel);
        d.shape.smem = (size_t)padded_elems(nel) * cbytes;
        d.shape.cluster = 1;
        const size_t strips = (p.dcy + ((size_t)1 << log2W) - 1) >> log2W;
        const size_t groups = step == 0 ? (size_t)p.N1 : (size_t)p.N2;
        d.shape.grid = dim3((unsigned)(groups * strips), (unsigned)p.batch, 1);
    }
    return true;
}

// Kernel attributes (dynamic shared memory limit, 16-CTA clusters) belong to
// the device's context: set them once per device and compute type.
template <class A>
static cudaError_t prepare_once()
{
    static std::mutex mu;
    static bool done[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return cudaSuccess;
    e = RowLaunch<A>::prepare();
    if (e == cudaSuccess) e = ColLaunch<A>::prepare();
    if (e == cudaSuccess) e = ColStepLaunch<A>::prepare();
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

static bool has_fixed(int prec, bool rows, const DimPlan &d)
{
    switch (prec) {
    case HPXFFT_PREC_F64:
        return rows ? RowLaunch<ArithFF>::has_fixed(d.L, d.log2W, d.C) : ColLaunch<ArithFF>::has_fixed(d.L, d.log2W, d.C);
    case HPXFFT_PREC_F32:
    case HPXFFT_PREC_BF16X3:
        return rows ? RowLaunch<ArithF32>::has_fixed(d.L, d.log2W, d.C)
                    : ColLaunch<ArithF32>::has_fixed(d.L, d.log2W, d.C);
    default: return false;
    }
}

// elements per thread (= largest radix) of the compile-time chains
static int fixed_ept(int prec) { return f32_storage(prec) ? ArithF32::kEPTFixed : ArithFF::kEPTFixed; }

// (Ls, R) of every pass of the compile-time chain for length L, in order
// (the same rule as FixedPasses: the largest radix, then the remainder)
static std::vector<std::pair<int, int>> fixed_chain(int L, int maxR)
{
    std::vector<std::pair<int, int>> v;
    for (int Ls = 1; Ls < L;) {
        const int R = fixed_radix(L, Ls, maxR);
        v.push_back({Ls, R});
        Ls *= R;
    }
    return v;
}

static cudaError_t prepare_tc_once()
{
    static std::mutex mu;
    static bool done[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return cudaSuccess;
    e = TcColStepLaunch::prepare();
    if (e == cudaSuccess) e = TcRowLaunch::prepare();
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

static cudaError_t prepare_prec(int prec)
{
    switch (prec) {
    case HPXFFT_PREC_F64: {
        cudaError_t e = prepare_once<ArithFF>();
        return e == cudaSuccess ? RowLaunchFF16::prepare() : e;
    }
    case HPXFFT_PREC_F64_NATIVE: return prepare_once<ArithF64>();
    case HPXFFT_PREC_BF16X3: {
        cudaError_t e = prepare_once<ArithF32>();
        return e == cudaSuccess ? prepare_tc_once() : e;
    }
    default: return prepare_once<ArithF32>();
    }
}

static cudaError_t gen_twiddles(int prec, void *tab, int n, cudaStream_t st)
{
    switch (prec) {
    case HPXFFT_PREC_F64: return TwiddleLaunch<ArithFF>::full(tab, n, st);
    case HPXFFT_PREC_F64_NATIVE: return TwiddleLaunch<ArithF64>::full(tab, n, st);
    default: return TwiddleLaunch<ArithF32>::full(tab, n, st);
    }
}

static cudaError_t gen_pass_twiddles(int prec, void *tab, int Ls, int R, cudaStream_t st)
{
    switch (prec) {
    case HPXFFT_PREC_F64: return TwiddleLaunch<ArithFF>::pass(tab, Ls, R, st);
    case HPXFFT_PREC_F64_NATIVE: return TwiddleLaunch<ArithF64>::pass(tab, Ls, R, st);
    default: return TwiddleLaunch<ArithF32>::pass(tab, Ls, R, st);
    }
}

// Allocate and fill the per-pass tables of the compile-time chain of length
// L with radices up to maxR.
static int chain_tables(hpxfft_plan_s &p, int L, int maxR, void **ptab, cudaStream_t st)
{
    const auto chain = fixed_chain(L, maxR);
    size_t entries = 0;
    for (auto &c : chain)
        if (c.first > 1) entries += (size_t)c.first * (c.second - 1);
    if (cudaMalloc(ptab, p.tw_elem * (entries ? entries : 1)) != cudaSuccess) {
        cudaGetLastError();
        return fail(HPXFFT_ERR_ALLOC, "pass twiddle table");
    }
    size_t off = 0;
    for (auto &c : chain) {
        if (c.first == 1) continue;
        cudaError_t e = gen_pass_twiddles(p.prec, (char *)*ptab + off * p.tw_elem, c.first, c.second, st);
        if (e != cudaSuccess) return cuda_fail(e, "pass twiddle generation");
        off += (size_t)c.first * (c.second - 1);
    }
    return HPXFFT_OK;
}

// Allocate and fill the per-pass tables when the dimension uses a fixed chain.
static int setup_fixed(hpxfft_plan_s &p, DimPlan &d, bool rows, cudaStream_t st, int step = 0)
{
    d.FL = 0;
    if (!(step ? has_fixed_step(p.prec, d) : has_fixed(p.prec, rows, d))) return HPXFFT_OK;
    const int rc = chain_tables(p, d.L, fixed_ept(p.prec), &d.ptab, st);
    if (rc != HPXFFT_OK) return rc;
    d.FL = d.L;
    if (!(step && p.prec == HPXFFT_PREC_BF16X3)) d.shape.threads = fixed_threads(d.L, d.log2W, fixed_ept(p.prec));
    return HPXFFT_OK;
}

static RowArgs row_args(const hpxfft_plan_s &p, const void *in, void *out, int adjoint)
{
    RowArgs a{};
    a.in = in;
    a.out = out;
    a.in_stride = (long long)p.ncol;
    a.out_stride = (long long)p.ncol;
    a.in_bstride = (long long)(p.nx * p.ncol);
    a.out_bstride = (long long)(p.nx * p.ncol);
    a.nrows = (int)p.nx;
    a.M = (int)p.M;
    a.log2W = p.row.log2W;
    a.adjoint = adjoint;
    a.pp = p.row.pp;
    a.tw = p.tw_row;
    a.Ltab = (int)(2 * p.M);
    a.ptab = p.row.ptab;
    a.pairs_out = 0;
    a.exp_out = nullptr;
    a.exp_bstride = (long long)p.nx;
    return a;
}

// the forward row arguments with the radix-16 chain's tables
static RowArgs row16_args(const hpxfft_plan_s &p, RowArgs a)
{
    a.ptab = p.row16_ptab;
    return a;
}

static ColArgs col_args(const hpxfft_plan_s &p, void *data)
{
    ColArgs a{};
    a.data = data;
    a.row_stride = (long long)p.ncol;
    a.bstride = (long long)(p.nx * p.ncol);
    a.nx = (int)p.nx;
    a.ncols = (int)p.dcy;
    a.log2W = p.col.log2W;
    a.pp = p.col.pp;
    a.tw = p.tw_col;
    a.Ltab = (int)p.nx;
    a.ptab = p.col.ptab;
    return a;
}

static int collect(hpxfft_plan_s &p);

// Events of the next timing slot; reads back the oldest slot when all are in flight.
static cudaEvent_t *next_slot(hpxfft_plan_s &p)
{
    if (p.next - p.done >= hpxfft_plan_s::kSlots) {
        const long long keep = p.next;
        p.next = p.done + 1;  // collect exactly the oldest slot
        collect(p);
        p.next = keep;
    }
    return p.kev[p.next % hpxfft_plan_s::kSlots];
}

static ColStepArgs colstep_args(const hpxfft_plan_s &p, int step, const void *in, void *out, bool pairs = false)
{
    const DimPlan &d = step == 0 ? p.colA : p.colB;
    ColStepArgs a{};
    a.in = in;
    a.out = out;
    a.row_stride = (long long)p.ncol;
    a.in_bstride = a.out_bstride = (long long)(p.nx * p.ncol);
    a.ncols = (int)p.dcy;
    a.strips = (int)((p.dcy + ((size_t)1 << d.log2W) - 1) >> d.log2W);
    if (step == 0) {  // rows g + N1 m -> rows g + N1 k, times W_nx^(g k)
        a.in_step = a.out_step = p.N1;
        a.in_gmul = a.out_gmul = 1;
        a.post = 1;
    } else {  // rows N1 g + m -> rows g + N2 k
        a.in_step = 1;
        a.in_gmul = p.N1;
        a.out_step = p.N2;
        a.out_gmul = 1;
        a.post = 0;
    }
    a.L = d.L;
    a.log2W = d.log2W;
    a.pp = d.pp;
    a.tw = p.tw_col;
    a.Ltab = (int)p.nx;
    a.ptab = d.ptab;
    a.block_offset = 0;
    a.grid_blocks = (int)d.shape.grid.x;
    a.warp_local = p.ff_warp_cols ? 1 : 0;
    if (pairs && step == 0) {  // per-row exponents of the row kernel
        a.pairs_in = a.pairs_out = 1;
        a.exp_in = p.exp_rows;
        a.exp_rmod = 1 << 30;
        a.exp_rmul = 1;
        a.exp_cshift = 30;
        a.exp_in_bstride = (long long)p.nx;
        a.exp_out = p.exp_step_a;
    } else if (pairs) {  // scratch row N1 g + m came from step A block (m, strip)
        const int strips_a = (int)((p.dcy + ((size_t)1 << p.colA.log2W) - 1) >> p.colA.log2W);
        a.pairs_in = 1;
        a.exp_in = p.exp_step_a;
        a.exp_rmod = p.N1;
        a.exp_rmul = strips_a;
        a.exp_cshift = p.colA.log2W;
        a.exp_in_bstride = (long long)p.colA.shape.grid.x;
    }
    return a;
}

// The column pass on `data`: one cluster kernel (in place) or steps A and B
// (step B writes `dst`, which may be `data`).
template <class A>
static cudaError_t run_columns(hpxfft_plan_s &p, void *data, int dir, void *dst)
{
    if (!p.col_two_step) return ColLaunch<A>::run(col_args(p, data), dir, p.col.shape, p.col.FL, p.stream);
    if (p.tc_cols) {
        cudaError_t e = TcColStepLaunch::run(colstep_args(p, 0, data, p.scratch), p.tc_dft, p.dev_error, dir,
                                             p.colA.shape.grid, p.stream);
        if (e != cudaSuccess) return e;
        if ((e = cudaEventRecord(p.kev[p.next % hpxfft_plan_s::kSlots][3], p.stream)) != cudaSuccess) return e;
        return TcColStepLaunch::run(colstep_args(p, 1, p.scratch, dst), p.tc_dft, p.dev_error, dir,
                                    p.colB.shape.grid, p.stream);
    }
    const bool pairs = p.ff_pairs && dir < 0;
    cudaError_t e =
        ColStepLaunch<A>::run(colstep_args(p, 0, data, p.scratch, pairs), dir, p.colA.shape, p.colA.FL, p.stream);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventRecord(p.kev[p.next % hpxfft_plan_s::kSlots][3], p.stream)) != cudaSuccess) return e;
    return ColStepLaunch<A>::run(colstep_args(p, 1, p.scratch, dst, pairs), dir, p.colB.shape, p.colB.FL, p.stream);
}

// Both steps of a two-step sub-plan q from `in` to `out` (batch strides of
// their own, q's row stride), with per-row factors on step A's input
// (rows past pre_rows read as zero) and on step B's output (rows past
// post_rows not written).
// With `exp` (float-float sub-plans), step A stores raw pairs and one
// exponent per block into exp, and step B reads them.
template <class A>
static cudaError_t run_steps_with(hpxfft_plan_s &q, const void *in, long long in_bs, void *out, long long out_bs,
                                  int dir, const void *pre, int pre_rows, const void *post, int post_rows, int conj,
                                  int *exp = nullptr)
{
    ColStepArgs sa = colstep_args(q, 0, in, q.scratch);
    sa.in_bstride = in_bs;
    sa.pre_tab = pre;
    sa.pre_rows = pre_rows;
    sa.tab_conj = conj;
    ColStepArgs sb = colstep_args(q, 1, q.scratch, out);
    sb.out_bstride = out_bs;
    sb.post_tab = post;
    sb.post_rows = post_rows;
    sb.tab_conj = conj;
    if (exp) {
        sa.pairs_out = 1;
        sa.exp_out = exp;
        sb.pairs_in = 1;
        sb.exp_in = exp;
        sb.exp_rmod = q.N1;  // scratch row N1 g + m came from step A block (m, strip)
        sb.exp_rmul = sa.strips;
        sb.exp_cshift = q.colA.log2W;
        sb.exp_in_bstride = (long long)q.colA.shape.grid.x;
    }
    cudaError_t e = ColStepLaunch<A>::run(sa, dir, q.colA.shape, q.colA.FL, q.stream);
    if (e != cudaSuccess) return e;
    return ColStepLaunch<A>::run(sb, dir, q.colB.shape, q.colB.FL, q.stream);
}

// Bluestein's convolution along the columns of `scr` (M rows of `width`
// complex values, the chirped input zero-padded): DFT_M, times the kernel's
// spectrum (conjugated for the inverse; fused into the forward pass's last
// step when the sub-plan has two), inverse DFT_M.
template <class A>
static cudaError_t alt_convolve(hpxfft_plan_s &p, AltAxis &a, void *scr, int dir)
{
    const int mode = alt_mode(p.prec);
    const long long w = (long long)a.width, bs = (long long)(a.M * a.width);
    const int M = (int)a.M, conj = dir > 0;
    if (a.fused) {
        cudaError_t e = run_steps_with<A>(*a.sub, scr, bs, scr, bs, -1, nullptr, 0, a.kernel, M, conj, a.exp_blocks);
        return e == cudaSuccess
                   ? run_steps_with<A>(*a.sub, scr, bs, scr, bs, +1, nullptr, 0, nullptr, 0, 0, a.exp_blocks)
                   : e;
    }
    cudaError_t e = run_columns<A>(*a.sub, scr, -1, scr);
    if (e == cudaSuccess)
        e = scale_rows(mode, scr, w, bs, scr, w, bs, a.kernel, conj, (long long)a.M, (long long)a.M, w, (int)p.batch,
                       p.stream);
    if (e == cudaSuccess) e = run_columns<A>(*a.sub, scr, +1, scr);
    return e;
}

// Columns outside the direct kernels' sizes, in place on `data`: chirp and
// zero-pad into the scratch array, convolve, chirp back (dir -1 forward,
// +1 the unnormalised inverse).
template <class A>
static cudaError_t run_alt_columns(hpxfft_plan_s &p, void *data, int dir)
{
    AltAxis &a = p.alt_col;
    a.sub->stream = p.stream;
    const int mode = alt_mode(p.prec);
    const long long dcy = (long long)p.dcy, dbs = (long long)(p.nx * p.dcy), sbs = (long long)(a.M * a.width);
    const int conj = dir > 0, nb = (int)p.batch;
    if (a.fused) {
        // chirp and zero-padding in step A's loads, the kernel's spectrum in
        // step B's stores, the chirp back in the inverse's step B (which
        // writes only the nx rows of `data`)
        const int L = (int)p.nx, M = (int)a.M;
        cudaError_t e =
            run_steps_with<A>(*a.sub, data, dbs, p.alt_buf, sbs, -1, a.chirp, L, a.kernel, M, conj, a.exp_blocks);
        return e == cudaSuccess ? run_steps_with<A>(*a.sub, p.alt_buf, sbs, data, dbs, +1, nullptr, 0, a.chirp, L,
                                                    conj, a.exp_blocks)
                                : e;
    }
    cudaError_t e = scale_rows(mode, data, dcy, dbs, p.alt_buf, dcy, sbs, a.chirp, conj, (long long)p.nx,
                               (long long)a.M, dcy, nb, p.stream);
    if (e == cudaSuccess) e = alt_convolve<A>(p, a, p.alt_buf, dir);
    if (e == cudaSuccess)
        e = scale_rows(mode, p.alt_buf, dcy, sbs, data, dcy, dbs, a.chirp, conj, (long long)p.nx, (long long)p.nx,
                       dcy, nb, p.stream);
    return e;
}

// Rows outside the direct kernels' sizes, forward, `in` to `out`: the packed
// rows transposed into the scratch array's columns (chirped and zero-padded
// for Bluestein), the length-h transforms along them, then the r2c split
// while transposing back.
template <class A>
static cudaError_t run_alt_rows(hpxfft_plan_s &p, const void *in, void *out)
{
    AltAxis &a = p.alt_row;
    a.sub->stream = p.stream;
    const int mode = alt_mode(p.prec);
    const long long dcy = (long long)p.dcy, dbs = (long long)(p.nx * p.dcy);
    const long long w = (long long)a.width, tbs = (long long)(a.M * a.width), h = (long long)p.M;
    const int nb = (int)p.batch;
    const void *chirp = a.bluestein ? a.chirp : nullptr;
    cudaError_t e = transpose_scaled(mode, in, dcy, dbs, (long long)p.nx, h, p.alt_buf, w, tbs, (long long)a.M, w,
                                     chirp, 0, 0, nb, p.stream);
    if (e == cudaSuccess)
        e = a.bluestein ? alt_convolve<A>(p, a, p.alt_buf, -1) : run_columns<A>(*a.sub, p.alt_buf, -1, p.alt_buf);
    if (e == cudaSuccess)
        e = r2c_split(mode, p.alt_buf, w, tbs, h, chirp, a.wtab, out, dcy, dbs, (long long)p.nx, nb, p.stream);
    return e;
}

// The c2r (or its adjoint) of rows outside the direct kernels' sizes, in
// place: the Hermitian merge while transposing into the scratch array, the
// inverse length-h transforms along its columns, the packed rows
// transposed back (pad reals zero).
template <class A>
static cudaError_t run_alt_rows_c2r(hpxfft_plan_s &p, void *data, int adjoint)
{
    AltAxis &a = p.alt_row;
    a.sub->stream = p.stream;
    const int mode = alt_mode(p.prec);
    const long long dcy = (long long)p.dcy, dbs = (long long)(p.nx * p.dcy);
    const long long w = (long long)a.width, tbs = (long long)(a.M * a.width), h = (long long)p.M;
    const int nb = (int)p.batch;
    const void *chirp = a.bluestein ? a.chirp : nullptr;
    cudaError_t e = c2r_merge(mode, data, dcy, dbs, (long long)p.nx, h, chirp, a.wtab, adjoint, p.alt_buf, w, tbs,
                              (long long)a.M, w, nb, p.stream);
    if (e == cudaSuccess)
        e = a.bluestein ? alt_convolve<A>(p, a, p.alt_buf, +1) : run_columns<A>(*a.sub, p.alt_buf, +1, p.alt_buf);
    if (e == cudaSuccess)
        e = transpose_scaled(mode, p.alt_buf, w, tbs, h, (long long)p.nx, data, dcy, dbs, (long long)p.nx, dcy, chirp,
                             1, 1, nb, p.stream);
    return e;
}

// Float-float rows of 16384 pairs from `in` to `out` in two kernels: the
// DFTs of their two halves (the column scratch holds them), then the
// radix-2 combination with the packed-real split (pairs and one exponent
// per row when pairs_out, else doubles).
static cudaError_t run_row_halves(hpxfft_plan_s &p, const void *in, void *out, int prefetch_in, int pairs_out,
                                  int *exp_out)
{
    constexpr int L = 8192;
    void *ybuf = p.scratch ? p.scratch : p.half_buf;
    RowArgs a = row_args(p, in, ybuf, 0);
    a.nrows = (int)(2 * p.nx);
    a.M = L;
    a.out_stride = 2LL * L;
    a.out_bstride = 2LL * L * 2 * (long long)p.nx;
    a.ptab = p.row16_ptab;
    a.pairs_out = 1;
    a.exp_out = p.half_exp;
    a.exp_bstride = 2LL * (long long)p.nx;
    a.prefetch = prefetch_in;
    cudaError_t e = RowLaunchFF16::halves(a, p.row16_shape, p.stream);
    if (e != cudaSuccess) return e;
    return combine_halves_split(ybuf, 2LL * L * (long long)p.nx, p.half_exp, 2LL * (long long)p.nx, L, p.half_wz,
                                p.half_ws, out, (long long)p.ncol, (long long)(p.nx * p.ncol), pairs_out, exp_out,
                                (long long)p.nx, (long long)p.nx, (int)p.batch, p.stream);
}

// Rows from `in` to `out`, columns on `out`; with the two-step column pass
// the last step writes `final_out` when it is given (the host buffer of the
// zero-copy path).
template <class A>
static cudaError_t run_forward(hpxfft_plan_s &p, const void *in, void *out, void *final_out = nullptr,
                               int prefetch_in = 1)
{
    cudaError_t e;
    cudaEvent_t *ev = next_slot(p);
    if ((e = cudaEventRecord(ev[0], p.stream)) != cudaSuccess) return e;
    RowArgs ra = row_args(p, in, out, 0);
    ra.prefetch = prefetch_in;
    if (p.ff_pairs) {
        ra.pairs_out = 1;
        ra.exp_out = p.exp_rows;
    }
    if (p.alt_row.on)
        e = run_alt_rows<A>(p, in, out);
    else if (p.row_halves)
        e = run_row_halves(p, in, out, prefetch_in, ra.pairs_out, ra.exp_out);
    else if (p.ff_row16)
        e = RowLaunchFF16::r2c(row16_args(p, ra), p.row16_shape, p.stream);
    else if (p.tc_rows)
        e = TcRowLaunch::run(ra, p.tc_dft, p.dev_error, p.row.shape.grid, p.stream);
    else
        e = RowLaunch<A>::r2c(ra, p.row.shape, p.row.FL, p.stream);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev[1], p.stream)) != cudaSuccess) return e;
    void *dst = final_out && p.col_two_step ? final_out : out;
    if ((e = p.alt_col.on ? run_alt_columns<A>(p, out, -1) : run_columns<A>(p, out, -1, dst)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(ev[2], p.stream)) != cudaSuccess) return e;
    ++p.next;
    return cudaSuccess;
}

template <class A>
static cudaError_t run_inverse(hpxfft_plan_s &p, void *data, int adjoint)
{
    cudaError_t e;
    cudaEvent_t *ev = next_slot(p);
    if ((e = cudaEventRecord(ev[0], p.stream)) != cudaSuccess) return e;
    if ((e = p.alt_col.on ? run_alt_columns<A>(p, data, +1) : run_columns<A>(p, data, +1, data)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(ev[1], p.stream)) != cudaSuccess) return e;
    e = p.alt_row.on ? run_alt_rows_c2r<A>(p, data, adjoint)
                     : RowLaunch<A>::c2r(row_args(p, data, data, adjoint), p.row.shape, p.row.FL, p.stream);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev[2], p.stream)) != cudaSuccess) return e;
    ++p.next;
    return cudaSuccess;
}

// Host buffer to host buffer with the transfers overlapped with the
// kernels (two-step column plans, one array).  The rows split into kChunks
// chunks by step A's groups: chunk c holds rows g + N1 m, g in [c G, (c+1) G)
// (G = N1 / kChunks), which one strided copy brings to the device; its row
// kernel and its step A blocks run while the next chunk is in flight.  Step
// B runs in chunks of its groups k2; chunk c completes output rows k2 + N2
// k1, which one strided copy takes back while step B works on the next
// chunk.  Returns false (nothing queued) when the plan has no such shape.
static bool pipelined_shape(const hpxfft_plan_s &p)
{
    const int K = hpxfft_plan_s::kChunks;
    return p.col_two_step && p.batch == 1 && !p.columns_only && !p.rows_only && !p.alt_row.on && !p.row_halves &&
           p.N1 % K == 0 && p.N2 % K == 0;
}

static cudaError_t ensure_pipeline(hpxfft_plan_s &p)
{
    if (p.copy_in) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&p.copy_in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p.copy_out, cudaStreamNonBlocking);
    for (int c = 0; c < hpxfft_plan_s::kChunks && e == cudaSuccess; ++c)
        for (cudaEvent_t *ev : {&p.chunk_in[c], &p.chunk_b[c], &p.chunk_out[c]})
            if (e == cudaSuccess) e = cudaEventCreate(ev);
    return e;
}

template <class A>
static cudaError_t run_forward_pipelined(hpxfft_plan_s &p, void *h)
{
    const int K = hpxfft_plan_s::kChunks;
    const size_t rb = p.ncol * p.real_bytes;  // bytes per row
    const int GA = p.N1 / K, GB = p.N2 / K;
    char *d = static_cast<char *>(p.dbuf);
    char *hc = static_cast<char *>(h);
    const bool pairs = p.ff_pairs;
    cudaError_t e;
    cudaEvent_t *ev = next_slot(p);
    if ((e = cudaEventRecord(ev[0], p.stream)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(p.copy_in, ev[0], 0)) != cudaSuccess) return e;
    for (int c = 0; c < K; ++c) {
        if ((e = cudaMemcpy2DAsync(d + c * GA * rb, p.N1 * rb, hc + c * GA * rb, p.N1 * rb, GA * rb, p.N2,
                                   cudaMemcpyHostToDevice, p.copy_in)) != cudaSuccess)
            return e;
        if ((e = cudaEventRecord(p.chunk_in[c], p.copy_in)) != cudaSuccess) return e;
    }
    const int wrows = 1 << p.row.log2W;
    const int stripsA = (int)((p.dcy + ((size_t)1 << p.colA.log2W) - 1) >> p.colA.log2W);
    const int stripsB = (int)((p.dcy + ((size_t)1 << p.colB.log2W) - 1) >> p.colB.log2W);
    for (int c = 0; c < K; ++c) {
        if ((e = cudaStreamWaitEvent(p.stream, p.chunk_in[c], 0)) != cudaSuccess) return e;
        // the chunk's rows as a strided batch: N2 items of GA consecutive
        // rows, N1 rows apart, starting at row c GA
        char *d0 = d + c * GA * rb;
        RowArgs ra = row_args(p, d0, d0, 0);
        ra.nrows = GA;
        ra.in_bstride = ra.out_bstride = (long long)p.N1 * (long long)p.ncol;
        ra.prefetch = 1;
        if (pairs) {
            ra.pairs_out = 1;
            ra.exp_out = p.exp_rows + c * GA;
            ra.exp_bstride = p.N1;
        }
        LaunchShape rs = p.row.shape;
        rs.grid = dim3((unsigned)(((GA + wrows - 1) / wrows) * p.row.C), (unsigned)p.N2, 1);
        if (p.ff_row16) {
            LaunchShape r16 = p.row16_shape;
            r16.grid = rs.grid;
            e = RowLaunchFF16::r2c(row16_args(p, ra), r16, p.stream);
        } else {
            e = p.tc_rows ? TcRowLaunch::run(ra, p.tc_dft, p.dev_error, rs.grid, p.stream)
                          : RowLaunch<A>::r2c(ra, rs, p.row.FL, p.stream);
        }
        if (e != cudaSuccess) return e;
        ColStepArgs aa = colstep_args(p, 0, d, p.scratch, pairs);
        aa.block_offset = c * GA * stripsA;
        LaunchShape as = p.colA.shape;
        as.grid = dim3((unsigned)(GA * stripsA), 1, 1);
        e = p.tc_cols ? TcColStepLaunch::run(aa, p.tc_dft, p.dev_error, -1, as.grid, p.stream)
                      : ColStepLaunch<A>::run(aa, -1, as, p.colA.FL, p.stream);
        if (e != cudaSuccess) return e;
    }
    if ((e = cudaEventRecord(ev[1], p.stream)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev[3], p.stream)) != cudaSuccess) return e;
    for (int c = 0; c < K; ++c) {
        ColStepArgs ba = colstep_args(p, 1, p.scratch, d, pairs);
        ba.block_offset = c * GB * stripsB;
        LaunchShape bs = p.colB.shape;
        bs.grid = dim3((unsigned)(GB * stripsB), 1, 1);
        e = p.tc_cols ? TcColStepLaunch::run(ba, p.tc_dft, p.dev_error, -1, bs.grid, p.stream)
                      : ColStepLaunch<A>::run(ba, -1, bs, p.colB.FL, p.stream);
        if (e != cudaSuccess) return e;
        if ((e = cudaEventRecord(p.chunk_b[c], p.stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(p.copy_out, p.chunk_b[c], 0)) != cudaSuccess) return e;
        if ((e = cudaMemcpy2DAsync(hc + c * GB * rb, p.N2 * rb, d + c * GB * rb, p.N2 * rb, GB * rb, p.N1,
                                   cudaMemcpyDeviceToHost, p.copy_out)) != cudaSuccess)
            return e;
        if ((e = cudaEventRecord(p.chunk_out[c], p.copy_out)) != cudaSuccess) return e;
    }
    if ((e = cudaEventRecord(ev[2], p.stream)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(p.stream, p.chunk_out[K - 1], 0)) != cudaSuccess) return e;
    ++p.next;
    return cudaSuccess;
}

static cudaError_t dispatch_forward_pipelined(hpxfft_plan_s &p, void *h)
{
    switch (p.prec) {
    case HPXFFT_PREC_F64: return run_forward_pipelined<ArithFF>(p, h);
    case HPXFFT_PREC_F64_NATIVE: return run_forward_pipelined<ArithF64>(p, h);
    default: return run_forward_pipelined<ArithF32>(p, h);
    }
}

// prefetch_in = 0 when `in` is host memory read over the host link
static cudaError_t dispatch_forward(hpxfft_plan_s &p, const void *in, void *out, void *final_out = nullptr,
                                   int prefetch_in = 1)
{
    switch (p.prec) {
    case HPXFFT_PREC_F64: return run_forward<ArithFF>(p, in, out, final_out, prefetch_in);
    case HPXFFT_PREC_F64_NATIVE: return run_forward<ArithF64>(p, in, out, final_out, prefetch_in);
    default: return run_forward<ArithF32>(p, in, out, final_out, prefetch_in);
    }
}

// The column pass alone, forward, in place (timed like a transform: the
// row slot of the timing ring is empty).
template <class A>
static cudaError_t run_columns_only(hpxfft_plan_s &p, void *data)
{
    cudaError_t e;
    cudaEvent_t *ev = next_slot(p);
    if ((e = cudaEventRecord(ev[0], p.stream)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev[1], p.stream)) != cudaSuccess) return e;
    if ((e = p.alt_col.on ? run_alt_columns<A>(p, data, -1) : run_columns<A>(p, data, -1, data)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(ev[2], p.stream)) != cudaSuccess) return e;
    ++p.next;
    return cudaSuccess;
}

// The row pass alone, forward, `in` to `out` (timed like a transform: the
// column slot of the timing ring is empty).  Doubles in and out for FP64.
template <class A>
static cudaError_t run_rows_only(hpxfft_plan_s &p, const void *in, void *out)
{
    cudaError_t e;
    cudaEvent_t *ev = next_slot(p);
    if ((e = cudaEventRecord(ev[0], p.stream)) != cudaSuccess) return e;
    RowArgs ra = row_args(p, in, out, 0);
    ra.prefetch = 1;
    e = p.alt_row.on    ? run_alt_rows<A>(p, in, out)
        : p.row_halves ? run_row_halves(p, in, out, 1, 0, nullptr)
        : p.ff_row16   ? RowLaunchFF16::r2c(row16_args(p, ra), p.row16_shape, p.stream)
                       : RowLaunch<A>::r2c(ra, p.row.shape, p.row.FL, p.stream);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev[1], p.stream)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev[2], p.stream)) != cudaSuccess) return e;
    ++p.next;
    return cudaSuccess;
}

static cudaError_t dispatch_rows_only(hpxfft_plan_s &p, const void *in, void *out)
{
    switch (p.prec) {
    case HPXFFT_PREC_F64: return run_rows_only<ArithFF>(p, in, out);
    case HPXFFT_PREC_F64_NATIVE: return run_rows_only<ArithF64>(p, in, out);
    default: return run_rows_only<ArithF32>(p, in, out);
    }
}

static cudaError_t dispatch_columns_only(hpxfft_plan_s &p, void *data)
{
    switch (p.prec) {
    case HPXFFT_PREC_F64: return run_columns_only<ArithFF>(p, data);
    case HPXFFT_PREC_F64_NATIVE: return run_columns_only<ArithF64>(p, data);
    default: return run_columns_only<ArithF32>(p, data);
    }
}

static cudaError_t dispatch_inverse(hpxfft_plan_s &p, void *data, int adjoint)
{
    switch (p.prec) {
    case HPXFFT_PREC_F64: return run_inverse<ArithFF>(p, data, adjoint);
    case HPXFFT_PREC_F64_NATIVE: return run_inverse<ArithF64>(p, data, adjoint);
    default: return run_inverse<ArithF32>(p, data, adjoint);
    }
}

// Read back every unread timing slot (blocks until those transforms are
// done).  The per-key measurements describe the most recent transform, like
// the reference's measurements_ map; the sums feed hpxfft_timing_stats.
static int collect(hpxfft_plan_s &p)
{
    const int K = hpxfft_plan_s::kSlots;
    for (; p.done < p.next; ++p.done) {
        cudaEvent_t *ev = p.kev[p.done % K];
        cudaError_t e = cudaEventSynchronize(ev[2]);
        if (e != cudaSuccess) return cuda_fail(e, "transform");
        float a = 0, b = 0, c = 0;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        cudaEventElapsedTime(&c, ev[0], ev[2]);
        p.sum_first += 1e-3 * a;
        p.sum_second += 1e-3 * b;
        p.sum_total += 1e-3 * c;
        if (p.col_two_step) {
            // forward: row, A, B (event 3 between A and B); inverse: A, B, row
            float sa = 0;
            cudaEventElapsedTime(&sa, ev[0], ev[3]);
            p.sum_step_a += 1e-3 * sa;
        }
        ++p.nsum;
        p.meas["first_fftw"] = 1e-3 * a;
        p.meas["first_trans"] = 0.0;
        p.meas["second_fftw"] = 1e-3 * b;
        p.meas["second_trans"] = 0.0;
        p.meas["total"] = 1e-3 * c;
        const double bytes = 4.0 * (double)(p.nx * p.dcy * 2 * p.real_bytes) * (double)p.batch;
        p.meas["gbps"] = c > 0 ? bytes / (1e-3 * c) / 1e9 : 0.0;
        const double n = (double)p.nx * (double)p.ny;
        p.meas["gflops"] = c > 0 && n > 1 ? 2.5 * n * std::log2(n) * (double)p.batch / (1e-3 * c) / 1e9 : 0.0;
        p.meas["roofline"] = p.peak_gbps > 0 ? p.meas["gbps"] / p.peak_gbps : 0.0;
        if (p.done + 1 == p.next && p.pending_copy) {
            float h = 0, d = 0, t = 0;
            cudaEventElapsedTime(&h, p.ev_copy[0], ev[0]);
            cudaEventElapsedTime(&d, ev[2], p.ev_copy[1]);
            cudaEventElapsedTime(&t, p.ev_copy[0], p.ev_copy[1]);
            p.meas["h2d"] = 1e-3 * h;
            p.meas["d2h"] = 1e-3 * d;
            p.meas["e2e"] = 1e-3 * t;
            p.meas["host_zero_copy"] = p.last_zero_copy ? 1.0 : 0.0;
            p.pending_copy = false;
        }
    }
    return HPXFFT_OK;
}

static bool valid_flag(const char *f)
{
    if (!f) return false;
    return !strcmp(f, "estimate") || !strcmp(f, "measure") || !strcmp(f, "patient") || !strcmp(f, "exhaustive");
}

static std::string describe(const hpxfft_plan_s &p, const DimPlan &d, const char *what, size_t len)
{
    char buf[512];
    std::string radices;
    for (int i = 0; i < d.pp.n; ++i) radices += (i ? "x" : "") + std::to_string(d.pp.radix[i]);
    if (radices.empty()) radices = "1";
    snprintf(buf, sizeof(buf),
             "(gpu-%s n=%zu cluster=%d local=%d radices=%s chain=%s interleaved=%d grid=%ux%u threads=%d smem=%zu "
             "precision=%s)",
             what, len, d.C, d.L, radices.c_str(), d.FL ? "compile-time" : "runtime", 1 << d.log2W, d.shape.grid.x,
             d.shape.grid.y, d.shape.threads, d.shape.smem,
             p.prec == HPXFFT_PREC_F64          ? "f64-floatfloat"
             : p.prec == HPXFFT_PREC_F64_NATIVE ? "f64-dfma"
             : p.prec == HPXFFT_PREC_BF16X3     ? ((&d == &p.row ? p.tc_rows : p.tc_cols) ? "bf16x3-tcgen05" : "f32")
                                                : "f32");
    return buf;
}

}  // namespace hpxfft_gpu

using namespace hpxfft_gpu;

extern "C" {

const char *hpxfft_status_string(int s)
{
    switch (s) {
    case HPXFFT_OK: return "ok";
    case HPXFFT_ERR_INVALID_ARG: return "invalid argument";
    case HPXFFT_ERR_UNSUPPORTED_SIZE: return "unsupported size";
    case HPXFFT_ERR_ALLOC: return "allocation failed";
    case HPXFFT_ERR_CUDA: return "CUDA error";
    case HPXFFT_ERR_TIMEOUT: return "device wait timed out";
    case HPXFFT_ERR_STATE: return "invalid state";
    case HPXFFT_ERR_IO: return "file I/O error";
    default: return "unknown status";
    }
}

const char *hpxfft_last_error(void) { return g_last_error.c_str(); }

int hpxfft_plan_flag_valid(const char *plan_flag) { return valid_flag(plan_flag) ? 1 : 0; }

}  // extern "C"

namespace hpxfft_gpu {

// Choices forced through the environment (tests and manual tuning):
// HPXFFT_COLUMNS=cluster|steps, HPXFFT_FF_PAIRS=0|1, HPXFFT_TC_VECTORS=256|512,
// HPXFFT_TC_ROWS=0|1.  They override the rules and the plan search, which
// then varies only the other choices.
static PlanChoice env_choice()
{
    PlanChoice c;
    if (const char *v = std::getenv("HPXFFT_COLUMNS")) {
        if (!strcmp(v, "cluster")) c.columns = 1;
        if (!strcmp(v, "steps")) c.columns = 2;
    }
    if (const char *v = std::getenv("HPXFFT_FF_PAIRS")) c.ff_pairs = !strcmp(v, "0") ? 0 : 1;
    if (const char *v = std::getenv("HPXFFT_TC_VECTORS")) c.tc_vectors = !strcmp(v, "512") ? 512 : 256;
    if (const char *v = std::getenv("HPXFFT_TC_ROWS")) c.tc_rows = !strcmp(v, "0") ? 0 : 1;
    return c;
}

static PlanChoice merged_choice(const PlanChoice &forced)
{
    PlanChoice c = forced;
    const PlanChoice env = env_choice();
    if (env.columns >= 0) c.columns = env.columns;
    if (env.ff_pairs >= 0) c.ff_pairs = env.ff_pairs;
    if (env.tc_vectors >= 0) c.tc_vectors = env.tc_vectors;
    if (env.tc_rows >= 0) c.tc_rows = env.tc_rows;
    return c;
}

}  // namespace hpxfft_gpu

static int create_plan_with(hpxfft_plan *out, size_t n_row, size_t n_col, size_t batch, int precision,
                            const char *plan_flag, int mode, const PlanChoice &forced, bool allow_alt = true);

// Longest n_row for rows outside the direct kernels' sizes (the transposing
// kernels tile n_row in 32-row tiles on one grid dimension with the others).
constexpr size_t kAltMaxRows = (size_t)1 << 21;

static int alt_sub_plan(hpxfft_plan_s &p, size_t len, size_t width, hpxfft_plan *sub)
{
    return create_plan_with(sub, len, 2 * width, p.batch, p.prec, "estimate", kPlanColumns, PlanChoice{}, false);
}

// Bluestein tables for a.L, a.M in the plan's arithmetic.
static int alt_tables(hpxfft_plan_s &p, AltAxis &a)
{
    cudaError_t e = bluestein_tables(a.L, a.M, alt_mode(p.prec), &a.chirp, &a.kernel);
    if (e != cudaSuccess) return cuda_fail(e, "Bluestein tables");
    const hpxfft_plan_s &q = *a.sub;
    a.fused = q.col_two_step && !q.tc_cols && p.prec != HPXFFT_PREC_F64_NATIVE;
    // pair exchange between the steps: compiled float-float step shapes
    if (a.fused && p.prec == HPXFFT_PREC_F64 && q.colA.FL && q.colB.FL && q.colA.L <= kColStepMaxPairL &&
        q.colB.L <= kColStepMaxPairL) {
        if (cudaMalloc(&a.exp_blocks, sizeof(int) * q.colA.shape.grid.x * q.batch) != cudaSuccess) {
            cudaGetLastError();
            return fail(HPXFFT_ERR_ALLOC, "exponent arrays");
        }
    }
    return HPXFFT_OK;
}

// Rows outside the direct kernels' sizes: the column kernels of length
// h = ny/2 on a transposed copy when such a plan exists, else Bluestein.
static int setup_alt_rows(hpxfft_plan_s &p)
{
    AltAxis &a = p.alt_row;
    a.L = p.M;
    a.width = (std::max<size_t>(p.nx, 2) + 3) / 4 * 4;  // 64-byte rows of the scratch array start aligned
    int rc = alt_sub_plan(p, a.L, a.width, &a.sub);
    if (rc == HPXFFT_OK) {
        a.M = a.L;
    } else if (rc == HPXFFT_ERR_UNSUPPORTED_SIZE) {
        a.bluestein = true;
        a.M = bluestein_length(a.L);
        if ((rc = alt_sub_plan(p, a.M, a.width, &a.sub)) != HPXFFT_OK) return rc;
        if ((rc = alt_tables(p, a)) != HPXFFT_OK) return rc;
    } else {
        return rc;
    }
    cudaError_t e = split_table(a.L, alt_mode(p.prec), &a.wtab);
    return e == cudaSuccess ? HPXFFT_OK : cuda_fail(e, "split twiddles");
}

// Columns outside the direct kernels' sizes: Bluestein over the dcy columns.
static int setup_alt_cols(hpxfft_plan_s &p)
{
    AltAxis &a = p.alt_col;
    a.L = p.nx;
    a.width = p.dcy;
    a.bluestein = true;
    a.M = bluestein_length(a.L);
    int rc = alt_sub_plan(p, a.M, a.width, &a.sub);
    return rc == HPXFFT_OK ? alt_tables(p, a) : rc;
}

static void free_alt(AltAxis &a)
{
    if (a.sub) {
        a.sub->stream = a.sub->own_stream;
        hpxfft_plan_destroy(a.sub);
    }
    cudaFree(a.chirp);
    cudaFree(a.kernel);
    cudaFree(a.wtab);
    cudaFree(a.exp_blocks);
    a = AltAxis{};
}

// mode kPlanColumns: a plan of the column pass alone (c2c along n_row of
// n_col/2 complex columns), the last axis of a 3D transform or the column
// slab of a slab decomposition; no row plan, no row twiddles, no
// float-float pair exchange.  kPlanRows: the row pass alone (FP32 rows for
// split-BF16), the local rows of a slab decomposition.  `forced` sets the
// tunable choices (-1: the rules); the environment overrides both.
// Dimensions outside the direct kernels' sizes take the paths of AltAxis
// (not for split-BF16, and not when allow_alt is false: the sub-plans of
// those paths).
static int create_plan_with(hpxfft_plan *out, size_t n_row, size_t n_col, size_t batch, int precision,
                            const char *plan_flag, int mode, const PlanChoice &forced, bool allow_alt)
{
    const bool columns_only = mode == kPlanColumns, rows_only = mode == kPlanRows;
    if (!out) return fail(HPXFFT_ERR_INVALID_ARG, "plan pointer is null");
    *out = nullptr;
    if (!valid_flag(plan_flag)) return fail(HPXFFT_ERR_INVALID_ARG, "Invalid FFTW plan flag string");
    if (precision < HPXFFT_PREC_F64 || precision > HPXFFT_PREC_BF16X3)
        return fail(HPXFFT_ERR_INVALID_ARG, "unknown precision");
    if (n_row == 0 || batch == 0) return fail(HPXFFT_ERR_INVALID_ARG, "empty array");
    if (n_col < 4 || n_col % 2) return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "n_col must be 2*(ny/2+1) with ny >= 2 even");
    if (n_row > (1u << 30) || n_col > (1u << 30) || batch > 65535)
        return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "dimension too large");
    // the split-BF16 column steps need nx = N1 * N2 with N1, N2 in
    // {32, 64, 128, 256}: the same condition plan_colsteps applies below,
    // checked here before anything touches the device
    if (precision == HPXFFT_PREC_BF16X3 && !rows_only && (n_row < 1024 || n_row > 65536 || (n_row & (n_row - 1))))
        return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "split-BF16 precision needs n_row a power of two in [1024, 65536]");
    const auto t0 = std::chrono::steady_clock::now();
    hpxfft_plan_s *p = new (std::nothrow) hpxfft_plan_s();
    if (!p) return fail(HPXFFT_ERR_ALLOC, "host allocation failed");
    p->nx = n_row;
    p->dcy = n_col / 2;     // loop.cpp:164
    p->ny = 2 * p->dcy - 2; // loop.cpp:165
    p->M = p->ny / 2;
    p->ncol = n_col;
    p->batch = batch;
    p->prec = precision;
    p->flag = plan_flag;
    p->real_bytes = f32_storage(precision) ? 4 : 8;
    p->tw_elem = f32_storage(precision) ? 8 : 16;
    p->columns_only = columns_only;
    p->rows_only = rows_only;
    if (const char *v = std::getenv("HPXFFT_FF_WARP_COLS")) p->ff_warp_cols = strcmp(v, "0") != 0;
    const PlanChoice want = merged_choice(forced);
    p->choice.tc_vectors = want.tc_vectors == 512 ? 512 : 256;
    const bool rows_ok = columns_only || plan_rows(*p);
    bool cols_ok = rows_only || plan_cols(*p);
    // power-of-two columns longer than a cluster holds: the two-kernel pass
    bool steps_only = false;
    if (!cols_ok && precision != HPXFFT_PREC_F64_NATIVE && precision != HPXFFT_PREC_BF16X3 && want.columns != 1 &&
        plan_colsteps(*p))
        cols_ok = steps_only = true;
    if (!rows_ok || !cols_ok) {
        if (!allow_alt || precision == HPXFFT_PREC_BF16X3 || (!rows_ok && n_row > kAltMaxRows)) {
            delete p;
            return fail(HPXFFT_ERR_UNSUPPORTED_SIZE,
                        allow_alt ? "sizes outside the direct kernels need a precision other than split-BF16 and "
                                    "n_row <= 2^21 for long or prime-factor rows"
                                  : "sizes must have no prime factor above 13 and fit the per-cluster shared memory");
        }
        p->alt_row.on = !rows_ok;
        p->alt_col.on = !cols_ok;
    }
    cudaError_t e = prepare_prec(precision);
    if (e != cudaSuccess) {
        delete p;
        return cuda_fail(e, "kernel attributes");
    }
    if ((e = cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete p;
        return cuda_fail(e, "stream");
    }
    p->stream = p->own_stream;
    for (auto &slot : p->kev)
        for (auto &ev : slot)
            if ((e = cudaEventCreate(&ev)) != cudaSuccess) {
                hpxfft_plan_destroy(p);
                return cuda_fail(e, "event");
            }
    for (auto &ev : p->ev_copy)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) {
            hpxfft_plan_destroy(p);
            return cuda_fail(e, "event");
        }
    const bool direct_rows = !columns_only && !p->alt_row.on, direct_cols = !rows_only && !p->alt_col.on;
    if ((direct_rows && cudaMalloc(&p->tw_row, p->tw_elem * 2 * p->M) != cudaSuccess) ||
        (direct_cols && cudaMalloc(&p->tw_col, p->tw_elem * p->nx) != cudaSuccess)) {
        hpxfft_plan_destroy(p);
        return fail(HPXFFT_ERR_ALLOC, "twiddle tables");
    }
    int rc = direct_rows ? setup_fixed(*p, p->row, true, p->stream) : HPXFFT_OK;
    // float-float rows of 8192 pairs: the radix-16 chain (16 x 16 x 16 x 2,
    // 512 threads at 128 registers) issues fewer instructions than the
    // radix-8 one (16384^2 rows 2.81 -> 2.72 ms); HPXFFT_FF_ROW16=0 keeps
    // the radix-8 chain (tests, tuning)
    if (rc == HPXFFT_OK && direct_rows && precision == HPXFFT_PREC_F64 && p->row.FL == 8192 && p->row.C == 1 &&
        p->row.log2W == 0) {
        const char *v = std::getenv("HPXFFT_FF_ROW16");
        if (!v || strcmp(v, "0") != 0) {
            rc = chain_tables(*p, 8192, ArithFF16::kEPTFixed, &p->row16_ptab, p->stream);
            p->row16_shape = p->row.shape;
            p->row16_shape.threads = fixed_threads(8192, 0, ArithFF16::kEPTFixed);
            p->ff_row16 = rc == HPXFFT_OK;
        }
    }
    // float-float rows of 16384 pairs (two-CTA clusters of 8192): the two
    // kernels of row_halves (32768^2 rows 24.7 -> see design notes);
    // HPXFFT_FF_ROW_HALVES=0 keeps the cluster kernel
    if (rc == HPXFFT_OK && direct_rows && precision == HPXFFT_PREC_F64 && p->row.FL == 8192 && p->row.C == 2 &&
        p->row.log2W == 0) {
        const char *v = std::getenv("HPXFFT_FF_ROW_HALVES");
        if (!v || strcmp(v, "0") != 0) {
            rc = chain_tables(*p, 8192, ArithFF16::kEPTFixed, &p->row16_ptab, p->stream);
            cudaError_t e2 = cudaSuccess;
            if (rc == HPXFFT_OK && cudaMalloc(&p->half_exp, sizeof(int) * 2 * p->nx * p->batch) != cudaSuccess) {
                cudaGetLastError();
                rc = fail(HPXFFT_ERR_ALLOC, "exponent arrays");
            }
            if (rc == HPXFFT_OK && ((e2 = split_table(8192, kTabFF, &p->half_wz)) != cudaSuccess ||
                                    (e2 = split_table(16384, kTabFF, &p->half_ws)) != cudaSuccess))
                rc = cuda_fail(e2, "row twiddles");
            p->row16_shape = p->row.shape;
            p->row16_shape.threads = fixed_threads(8192, 0, ArithFF16::kEPTFixed);
            p->row16_shape.cluster = 1;
            p->row16_shape.grid = dim3((unsigned)(2 * p->nx), (unsigned)p->batch, 1);
            p->row_halves = rc == HPXFFT_OK;
        }
    }
    if (rc == HPXFFT_OK && direct_cols && !steps_only) rc = setup_fixed(*p, p->col, false, p->stream);
    // column strategy: the two-kernel pass streams 512-byte row segments and
    // wins once the cluster kernel needs 8 or more CTAs per strip (the rule;
    // the plan's choice may set either)
    bool want_steps = steps_only || (direct_cols && p->col.C >= 8);
    if (want.columns == 1 && !steps_only) want_steps = false;
    if (want.columns == 2 && direct_cols) want_steps = true;
    if (rows_only) want_steps = false;
    if (precision == HPXFFT_PREC_BF16X3 && !rows_only) {
        // the tensor-core stage lives in the column steps: nx = N1 * N2 with
        // N1, N2 in {32, 64, 128, 256}
        if (rc == HPXFFT_OK && !plan_colsteps(*p)) {
            hpxfft_plan_destroy(p);
            return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "split-BF16 precision needs n_row a power of two in [1024, 65536]");
        }
        want_steps = true;
        if (rc == HPXFFT_OK) {
            if (cudaMalloc(&p->tc_dft, TcColStepLaunch::table_bytes()) != cudaSuccess ||
                cudaMalloc(&p->dev_error, sizeof(int)) != cudaSuccess) {
                cudaGetLastError();
                rc = fail(HPXFFT_ERR_ALLOC, "tensor-core tables");
            } else if ((e = TcColStepLaunch::table(p->tc_dft, p->stream)) != cudaSuccess ||
                       (e = cudaMemsetAsync(p->dev_error, 0, sizeof(int), p->stream)) != cudaSuccess) {
                rc = cuda_fail(e, "tensor-core tables");
            } else {
                p->tc_cols = true;
                // rows: the tensor-core r2c where the FP32 plan has a compiled
                // single-CTA shape of 128..512 vectors; other rows stay FP32
                // (the launcher sizes its own CTAs; row.shape stays the FP32
                // one, which the inverse's c2r rows use) when the choice
                // tc_rows = 1 asks for them.  The rule keeps FP32 rows:
                // 16384^2 rows take 0.54 ms in FP32 against 0.87 ms on the
                // tensor cores, whose BF16 split costs more CUDA-core work
                // than the radix-16 butterfly it replaces (the whole
                // transform: 1.66 against 1.98 ms)
                if (!columns_only && p->row.FL && TcRowLaunch::supports((int)p->M, p->row.log2W, p->row.C) &&
                    want.tc_rows == 1)
                    p->tc_rows = true;
            }
        }
    }
    if (rc == HPXFFT_OK && precision != HPXFFT_PREC_F64_NATIVE && want_steps && plan_colsteps(*p)) {
        rc = setup_fixed(*p, p->colA, false, p->stream, 1);
        if (rc == HPXFFT_OK) rc = setup_fixed(*p, p->colB, false, p->stream, 2);
        if (rc == HPXFFT_OK) {
            if (cudaMalloc(&p->scratch, p->nx * p->ncol * p->real_bytes * p->batch) != cudaSuccess) {
                cudaGetLastError();
                rc = fail(HPXFFT_ERR_ALLOC, "column scratch buffer");
            } else {
                p->col_two_step = true;
            }
        }
    }
    if (rc == HPXFFT_OK && steps_only && !p->col_two_step)
        rc = fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "no column plan for this n_row");
    // float-float pair exchange between the forward kernels (compiled step
    // shapes only); the choice ff_pairs = 0 keeps doubles in between
    if (rc == HPXFFT_OK && direct_rows && precision == HPXFFT_PREC_F64 && p->col_two_step && p->colA.FL && p->colB.FL &&
        p->colA.L <= kColStepMaxPairL && p->colB.L <= kColStepMaxPairL && want.ff_pairs != 0) {
        if (cudaMalloc(&p->exp_rows, sizeof(int) * p->nx * p->batch) != cudaSuccess ||
            cudaMalloc(&p->exp_step_a, sizeof(int) * p->colA.shape.grid.x * p->batch) != cudaSuccess) {
            cudaGetLastError();
            rc = fail(HPXFFT_ERR_ALLOC, "exponent arrays");
        } else {
            p->ff_pairs = true;
        }
    }
    if (rc == HPXFFT_OK && p->row_halves && !p->scratch &&
        cudaMalloc(&p->half_buf, sizeof(double) * 2 * 16384 * p->nx * p->batch) != cudaSuccess) {
        cudaGetLastError();
        rc = fail(HPXFFT_ERR_ALLOC, "row buffer");
    }
    if (rc != HPXFFT_OK) {
        std::string msg = g_last_error;
        hpxfft_plan_destroy(p);
        return fail(rc, msg);
    }
    if ((direct_rows && (e = gen_twiddles(precision, p->tw_row, (int)(2 * p->M), p->stream)) != cudaSuccess) ||
        (direct_cols && (e = gen_twiddles(precision, p->tw_col, (int)p->nx, p->stream)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(p->stream)) != cudaSuccess) {
        hpxfft_plan_destroy(p);
        return cuda_fail(e, "twiddle generation");
    }
    // the sub-plans, tables and scratch array of the other paths
    if (p->alt_row.on) rc = setup_alt_rows(*p);
    if (rc == HPXFFT_OK && p->alt_col.on) rc = setup_alt_cols(*p);
    if (rc == HPXFFT_OK && (p->alt_row.on || p->alt_col.on)) {
        const size_t cr = p->alt_row.on ? p->alt_row.M * p->alt_row.width : 0;
        const size_t cc = p->alt_col.on ? p->alt_col.M * p->alt_col.width : 0;
        if (cudaMalloc(&p->alt_buf, std::max(cr, cc) * 2 * p->real_bytes * p->batch) != cudaSuccess) {
            cudaGetLastError();
            rc = fail(HPXFFT_ERR_ALLOC, "scratch array");
        }
    }
    if (rc != HPXFFT_OK) {
        std::string msg = g_last_error;
        hpxfft_plan_destroy(p);
        return fail(rc, msg);
    }
    {
        int dev = 0, clock_khz = 0, bus_bits = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&clock_khz, cudaDevAttrMemoryClockRate, dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&bus_bits, cudaDevAttrGlobalMemoryBusWidth, dev) == cudaSuccess)
            p->peak_gbps = 2.0 * clock_khz * 1e3 * (bus_bits / 8.0) / 1e9;  // double data rate
        cudaGetLastError();
    }
    const auto t1 = std::chrono::steady_clock::now();
    p->meas["plan"] = std::chrono::duration<double>(t1 - t0).count();
    // loop.cpp:188 counts dim_r_y r2c plans and dim_c_x c2c plans; keep that
    // formula for the key, with 2.5 n log2 n per r2c and 5 n log2 n per c2c
    const double ny = (double)p->ny, nx = (double)p->nx;
    const double f_r2c = 2.5 * ny * std::log2(ny), f_c2c = nx > 1 ? 5.0 * nx * std::log2(nx) : 0.0;
    p->meas["plan_flops"] = ny * f_r2c + nx * f_c2c;
    p->meas["plan_flops_actual"] = (nx * f_r2c + (double)p->dcy * f_c2c) * (double)batch;
    // which path each pass takes: Bluestein's convolution length (0: none),
    // rows on a transposed copy (1) or in the row kernel (0)
    p->meas["bluestein_rows"] = p->alt_row.bluestein ? (double)p->alt_row.M : 0.0;
    p->meas["bluestein_columns"] = p->alt_col.bluestein ? (double)p->alt_col.M : 0.0;
    p->meas["transposed_rows"] = p->alt_row.on ? 1.0 : 0.0;
    // the choices in effect
    p->choice.columns = p->col_two_step ? 2 : 1;
    p->choice.ff_pairs = p->ff_pairs ? 1 : 0;
    p->choice.tc_rows = p->tc_rows ? 1 : 0;
    if (!p->tc_cols) p->choice.tc_vectors = 0;
    p->tuned_from = "rules";
    *out = p;
    return HPXFFT_OK;
}

// ------------------------------------------------------------ plan search
// "estimate" plans by the fixed rules.  "measure", "patient" and
// "exhaustive" time every distinct candidate plan (column strategy,
// float-float pair exchange, split-BF16 vectors per CTA and tensor-core
// rows) on scratch arrays of the plan's size, keep the fastest and cache the
// choice under (shape, batch, precision, device architecture); the cache is
// written to and read from wisdom files with the batch plans'.  This is the
// planner step of fftw_adapter::{r2c_1d,c2c_1d}::plan
// (core/src/util/adapter_fftw.cpp:6-10,24-30) with FFTW_MEASURE and stronger
// (core/include/hpxfft/util/adapter_fftw.hpp:13-44), which run trial
// transforms on a scratch row (core/src/shared/loop.cpp:169-182).
namespace hpxfft_gpu {

// HPXFFT_ERR_TIMEOUT (and clears the flag) when a tensor-core kernel's wait gave up
static int check_device_error(hpxfft_plan p)
{
    if (!p->dev_error) return HPXFFT_OK;
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, p->dev_error, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "error flag");
    if (!flag) return HPXFFT_OK;
    cudaMemsetAsync(p->dev_error, 0, sizeof(int), p->stream);
    return fail(HPXFFT_ERR_TIMEOUT, "tensor-core MMA completion wait timed out");
}

static std::mutex g_choice_mu;
static std::map<std::string, PlanChoice> g_choices;

static std::string choice_key(size_t n_row, size_t n_col, size_t batch, int prec, int mode)
{
    int dev = 0, major = 0, minor = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev))
        cudaGetLastError();
    char buf[160];
    snprintf(buf, sizeof(buf), "2d;p%d;%zux%zu;b%zu;%s;sm%d%d", prec, n_row, n_col, batch,
             mode == kPlanColumns ? "cols" : mode == kPlanRows ? "rows" : "full",
             major, minor);
    return buf;
}

std::string describe_choice(const PlanChoice &c)
{
    std::string d = c.columns == 2 ? "columns=steps" : "columns=cluster";
    if (c.columns == 2) d += " ff_pairs=" + std::to_string(c.ff_pairs);
    if (c.tc_vectors > 0) d += " tc_vectors=" + std::to_string(c.tc_vectors) + " tc_rows=" + std::to_string(c.tc_rows);
    return d;
}

template <class S>
__global__ void tune_fill_kernel(S *p, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        unsigned h = (unsigned)(i * 2654435761u) ^ (unsigned)(i >> 32) ^ 0x9e3779b9u;
        h ^= h >> 16;
        h *= 0x7feb352du;
        h ^= h >> 15;
        p[i] = (S)((float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f);  // uniform[-1, 1)
    }
}

// Best time (ms) of `reps` transforms of plan q from `in` to `out` after one warm-up.
static double time_candidate(hpxfft_plan q, const void *in, void *out, int reps)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        return -1.0;
    }
    double best = -1.0;
    for (int r = 0; r <= reps; ++r) {
        if (cudaMemcpyAsync(out, in, q->nx * q->ncol * q->real_bytes * q->batch, cudaMemcpyDeviceToDevice,
                            q->stream) != cudaSuccess)
            break;
        cudaEventRecord(e0, q->stream);
        cudaError_t e = q->columns_only ? dispatch_columns_only(*q, out)
                        : q->rows_only  ? dispatch_rows_only(*q, in, out)
                                        : dispatch_forward(*q, in, out);
        cudaEventRecord(e1, q->stream);
        if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
            best = -1.0;
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && (best < 0 || ms < best)) best = ms;
    }
    cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (collect(*q) != HPXFFT_OK || check_device_error(q) != HPXFFT_OK) return -1.0;
    return best;
}

// Forget what the trial runs left in a plan's measurements and timing sums.
static void clear_trial_state(hpxfft_plan q)
{
    collect(*q);
    q->sum_first = q->sum_second = q->sum_total = q->sum_step_a = 0.0;
    q->nsum = 0;
    std::map<std::string, double> keep;
    for (const char *k : {"plan", "plan_flops", "plan_flops_actual", "bluestein_rows", "bluestein_columns",
                          "transposed_rows"})
        keep[k] = q->meas[k];
    q->meas.swap(keep);
}

}  // namespace hpxfft_gpu

static int create_plan(hpxfft_plan *out, size_t n_row, size_t n_col, size_t batch, int precision,
                       const char *plan_flag, int mode)
{
    if (!valid_flag(plan_flag) || !strcmp(plan_flag, "estimate"))
        return create_plan_with(out, n_row, n_col, batch, precision, plan_flag, mode, PlanChoice{});
    const auto t0 = std::chrono::steady_clock::now();
    auto finish = [&](hpxfft_plan q, const char *from) {
        q->flag = plan_flag;
        q->tuned_from = from;
        q->meas["plan"] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        q->meas["cached_plan"] = !strcmp(from, "wisdom") ? 1.0 : 0.0;
        q->meas["autotune_candidates"] = (double)q->tuning.size();
        q->meas["choice_columns"] = q->choice.columns;
        q->meas["choice_ff_pairs"] = q->choice.ff_pairs;
        q->meas["choice_tc_vectors"] = q->choice.tc_vectors;
        q->meas["choice_tc_rows"] = q->choice.tc_rows;
        *out = q;
        return HPXFFT_OK;
    };
    const std::string key = choice_key(n_row, n_col, batch, precision, mode);
    {
        PlanChoice cached;
        bool hit = false;
        {
            std::lock_guard<std::mutex> lock(g_choice_mu);
            auto it = g_choices.find(key);
            if (it != g_choices.end()) cached = it->second, hit = true;
        }
        if (hit) {
            hpxfft_plan q = nullptr;
            int rc = create_plan_with(&q, n_row, n_col, batch, precision, "estimate", mode, cached);
            if (rc != HPXFFT_OK) return rc;
            return finish(q, "wisdom");
        }
    }
    // candidates: every combination of the choices this precision has, less
    // those the environment fixes; plans that come out identical are timed once
    const PlanChoice env = env_choice();
    std::vector<int> cols = env.columns >= 0 ? std::vector<int>{env.columns} : std::vector<int>{2, 1};
    std::vector<int> pairs{-1}, vecs{-1}, trows{-1};
    if (precision == HPXFFT_PREC_F64 && env.ff_pairs < 0) pairs = {1, 0};
    if (precision == HPXFFT_PREC_BF16X3) {
        if (env.tc_vectors < 0) vecs = {256, 512};
        if (env.tc_rows < 0) trows = {1, 0};
    }
    const int reps = !strcmp(plan_flag, "measure") ? 3 : !strcmp(plan_flag, "patient") ? 5 : 10;
    std::vector<hpxfft_plan> plans;
    std::vector<std::string> seen;
    int first_rc = HPXFFT_OK;
    std::string first_msg;
    for (int c : cols)
        for (int fp : pairs)
            for (int nv : vecs)
                for (int tr : trows) {
                    PlanChoice cand;
                    cand.columns = c;
                    cand.ff_pairs = fp;
                    cand.tc_vectors = nv;
                    cand.tc_rows = tr;
                    hpxfft_plan q = nullptr;
                    int rc = create_plan_with(&q, n_row, n_col, batch, precision, "estimate", mode, cand);
                    if (rc != HPXFFT_OK) {
                        if (first_rc == HPXFFT_OK) first_rc = rc, first_msg = g_last_error;
                        continue;
                    }
                    const std::string d = describe_choice(q->choice);
                    if (std::find(seen.begin(), seen.end(), d) != seen.end()) {
                        hpxfft_plan_destroy(q);
                        continue;
                    }
                    seen.push_back(d);
                    plans.push_back(q);
                }
    if (plans.empty()) return fail(first_rc == HPXFFT_OK ? HPXFFT_ERR_UNSUPPORTED_SIZE : first_rc, first_msg);
    size_t best = 0;
    std::vector<double> ms(plans.size(), -1.0);
    if (plans.size() > 1) {
        // trial arrays of the plan's size, filled with uniform[-1, 1) values
        const size_t bytes = n_row * n_col * plans[0]->real_bytes * batch;
        void *bin = nullptr, *bout = nullptr;
        if (cudaMalloc(&bin, bytes) == cudaSuccess && cudaMalloc(&bout, bytes) == cudaSuccess) {
            if (plans[0]->real_bytes == 8)
                tune_fill_kernel<double><<<1024, 256, 0, plans[0]->stream>>>((double *)bin, bytes / 8);
            else
                tune_fill_kernel<float><<<1024, 256, 0, plans[0]->stream>>>((float *)bin, bytes / 4);
            cudaStreamSynchronize(plans[0]->stream);
            for (size_t i = 0; i < plans.size(); ++i) ms[i] = time_candidate(plans[i], bin, bout, reps);
            for (size_t i = 0; i < plans.size(); ++i)
                if (ms[i] >= 0 && (ms[best] < 0 || ms[i] < ms[best])) best = i;
        }
        cudaGetLastError();
        cudaFree(bin);
        cudaFree(bout);
    }
    for (size_t i = 0; i < plans.size(); ++i)
        if (i != best) hpxfft_plan_destroy(plans[i]);
    hpxfft_plan q = plans[best];
    clear_trial_state(q);
    if (plans.size() > 1 && ms[best] >= 0) {
        for (size_t i = 0; i < seen.size(); ++i) q->tuning.push_back({seen[i], ms[i]});
        q->meas["autotune_best_ms"] = ms[best];
        q->meas["autotune_chosen"] = (double)best;
        for (size_t i = 0; i < ms.size(); ++i) q->meas["autotune_ms_" + std::to_string(i)] = ms[i];
    }
    {
        std::lock_guard<std::mutex> lock(g_choice_mu);
        g_choices[key] = q->choice;
    }
    return finish(q, plans.size() > 1 ? "search" : "rules");
}

// wisdom of the 2D plans (the batch plans' entries are written by batch.cu)
namespace hpxfft_gpu {

void wisdom2d_write(FILE *f)
{
    std::lock_guard<std::mutex> lock(g_choice_mu);
    for (auto &kv : g_choices)
        fprintf(f, "%s %d %d %d %d\n", kv.first.c_str(), kv.second.columns, kv.second.ff_pairs, kv.second.tc_vectors,
                kv.second.tc_rows);
}

// One entry "2d;... columns ff_pairs tc_vectors tc_rows"; false if malformed.
bool wisdom2d_check(const std::string &key, const std::vector<long long> &v)
{
    return key.rfind("2d;", 0) == 0 && v.size() == 4 && (v[0] == 1 || v[0] == 2) && (v[1] == 0 || v[1] == 1) &&
           (v[2] == 0 || v[2] == 256 || v[2] == 512) && (v[3] == 0 || v[3] == 1);
}

void wisdom2d_add(const std::string &key, const std::vector<long long> &v)
{
    PlanChoice c;
    c.columns = (int)v[0];
    c.ff_pairs = (int)v[1];
    c.tc_vectors = (int)v[2];
    c.tc_rows = (int)v[3];
    std::lock_guard<std::mutex> lock(g_choice_mu);
    g_choices[key] = c;
}

void wisdom2d_forget()
{
    std::lock_guard<std::mutex> lock(g_choice_mu);
    g_choices.clear();
}

}  // namespace hpxfft_gpu

extern "C" {

int hpxfft_plan_create(hpxfft_plan *out, size_t n_row, size_t n_col, size_t batch, int precision,
                       const char *plan_flag)
{
    return create_plan(out, n_row, n_col, batch, precision, plan_flag, kPlanFull);
}

// ------------------------------------------------------------------ 3D r2c
// n0 x n1 x n2 reals, last axis padded to n_col = 2 (n2/2 + 1):  a batched
// 2D r2c over the n0 slabs (rows along axis 2, columns along axis 1), then
// the column pass along axis 0 over the n1 (n2/2 + 1) complex columns of
// the slab-major layout (rows of n1 n_col reals).
struct hpxfft_plan3d_s {
    hpxfft_plan slabs = nullptr;
    hpxfft_plan axis0 = nullptr;
    size_t n0 = 0, n1 = 0, ncol = 0, batch = 1;
};

int hpxfft_plan3d_create(hpxfft_plan3d *out, size_t n0, size_t n1, size_t n_col, size_t batch, int precision,
                         const char *plan_flag)
{
    if (!out) return fail(HPXFFT_ERR_INVALID_ARG, "plan pointer is null");
    *out = nullptr;
    if (n0 == 0 || n1 == 0 || batch == 0) return fail(HPXFFT_ERR_INVALID_ARG, "empty array");
    if (n0 * batch > 65535) return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "n0 * batch must not exceed 65535");
    if (n1 * n_col > (1u << 30)) return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "dimension too large");
    hpxfft_plan3d_s *p = new (std::nothrow) hpxfft_plan3d_s();
    if (!p) return fail(HPXFFT_ERR_ALLOC, "host allocation failed");
    p->n0 = n0;
    p->n1 = n1;
    p->ncol = n_col;
    p->batch = batch;
    int rc = create_plan(&p->slabs, n1, n_col, n0 * batch, precision, plan_flag, kPlanFull);
    if (rc == HPXFFT_OK) rc = create_plan(&p->axis0, n0, n1 * n_col, batch, precision, plan_flag, kPlanColumns);
    if (rc != HPXFFT_OK) {
        std::string msg = g_last_error;
        hpxfft_plan3d_destroy(p);
        return fail(rc, msg);
    }
    p->axis0->stream = p->slabs->stream;  // one stream orders both passes
    *out = p;
    return HPXFFT_OK;
}

int hpxfft_plan3d_destroy(hpxfft_plan3d p)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (p->axis0) {
        p->axis0->stream = p->axis0->own_stream;
        hpxfft_plan_destroy(p->axis0);
    }
    if (p->slabs) hpxfft_plan_destroy(p->slabs);
    delete p;
    return HPXFFT_OK;
}

int hpxfft_plan3d_set_stream(hpxfft_plan3d p, void *stream)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    p->slabs->stream = (cudaStream_t)stream;
    p->axis0->stream = (cudaStream_t)stream;
    return HPXFFT_OK;
}

int hpxfft_plan3d_buffer_bytes(hpxfft_plan3d p, size_t *bytes)
{
    if (!p || !bytes) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    *bytes = p->n0 * p->n1 * p->ncol * p->slabs->real_bytes * p->batch;
    return HPXFFT_OK;
}

int hpxfft_execute3d_r2c(hpxfft_plan3d p, void *d)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (!d) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    if ((uintptr_t)d & 15) return fail(HPXFFT_ERR_INVALID_ARG, "buffers must be 16-byte aligned");
    cudaError_t e = dispatch_forward(*p->slabs, d, d);
    if (e == cudaSuccess) e = dispatch_columns_only(*p->axis0, d);
    if (e != cudaSuccess) return cuda_fail(e, "3D forward launch");
    return HPXFFT_OK;
}

int hpxfft_plan3d_get_measurement(hpxfft_plan3d p, const char *name, double *value)
{
    if (!p || !name || !value) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    double a = 0, b = 0, c = 0;
    int rc = hpxfft_get_measurement(p->slabs, "first_fftw", &a);
    if (rc == HPXFFT_OK) rc = hpxfft_get_measurement(p->slabs, "second_fftw", &b);
    if (rc == HPXFFT_OK) rc = hpxfft_get_measurement(p->axis0, "total", &c);
    if (rc != HPXFFT_OK) return rc;
    if (!strcmp(name, "total"))
        *value = a + b + c;
    else if (!strcmp(name, "first_fftw"))
        *value = a;  // rows (axis 2)
    else if (!strcmp(name, "second_fftw"))
        *value = b;  // axis 1
    else if (!strcmp(name, "third_fftw"))
        *value = c;  // axis 0
    else
        return hpxfft_get_measurement(p->slabs, name, value);
    return HPXFFT_OK;
}

int hpxfft_plan_destroy(hpxfft_plan p)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (p->stream) cudaStreamSynchronize(p->stream);
    cudaFree(p->tw_row);
    cudaFree(p->tw_col);
    cudaFree(p->row.ptab);
    cudaFree(p->row16_ptab);
    cudaFree(p->half_exp);
    cudaFree(p->half_buf);
    cudaFree(p->half_wz);
    cudaFree(p->half_ws);
    cudaFree(p->col.ptab);
    cudaFree(p->colA.ptab);
    cudaFree(p->colB.ptab);
    cudaFree(p->scratch);
    cudaFree(p->dbuf);
    cudaFree(p->tc_dft);
    cudaFree(p->dev_error);
    cudaFree(p->exp_rows);
    cudaFree(p->exp_step_a);
    free_alt(p->alt_row);
    free_alt(p->alt_col);
    cudaFree(p->alt_buf);
    for (auto &slot : p->kev)
        for (auto &ev : slot)
            if (ev) cudaEventDestroy(ev);
    for (auto &ev : p->ev_copy)
        if (ev) cudaEventDestroy(ev);
    for (int c = 0; c < hpxfft_plan_s::kChunks; ++c)
        for (cudaEvent_t ev : {p->chunk_in[c], p->chunk_b[c], p->chunk_out[c]})
            if (ev) cudaEventDestroy(ev);
    if (p->copy_in) cudaStreamDestroy(p->copy_in);
    if (p->copy_out) cudaStreamDestroy(p->copy_out);
    if (p->own_stream) cudaStreamDestroy(p->own_stream);
    delete p;
    return HPXFFT_OK;
}

int hpxfft_plan_set_stream(hpxfft_plan p, void *stream)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    p->stream = (cudaStream_t)stream;  // verbatim: NULL is the legacy default stream
    return HPXFFT_OK;
}

int hpxfft_plan_get_stream(hpxfft_plan p, void **stream)
{
    if (!p || !stream) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    *stream = (void *)p->stream;
    return HPXFFT_OK;
}

int hpxfft_plan_buffer_bytes(hpxfft_plan p, size_t *bytes)
{
    if (!p || !bytes) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    *bytes = p->nx * p->ncol * p->real_bytes * p->batch;
    return HPXFFT_OK;
}

int hpxfft_execute_r2c_oop(hpxfft_plan p, const void *d_in, void *d_out)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (!d_in || !d_out) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    if (((uintptr_t)d_in | (uintptr_t)d_out) & 15) return fail(HPXFFT_ERR_INVALID_ARG, "buffers must be 16-byte aligned");
    cudaError_t e = dispatch_forward(*p, d_in, d_out);
    if (e != cudaSuccess) return cuda_fail(e, "forward launch");
    return HPXFFT_OK;
}

int hpxfft_execute_r2c(hpxfft_plan p, void *d) { return hpxfft_execute_r2c_oop(p, d, d); }

static int ensure_dbuf(hpxfft_plan p)
{
    size_t bytes = p->nx * p->ncol * p->real_bytes * p->batch;
    if (p->dbuf && p->dbuf_bytes >= bytes) return HPXFFT_OK;
    cudaFree(p->dbuf);
    p->dbuf = nullptr;
    if (cudaMalloc(&p->dbuf, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(HPXFFT_ERR_ALLOC, "device buffer");
    }
    p->dbuf_bytes = bytes;
    return HPXFFT_OK;
}


// Device address of a page-locked (pinned or registered) host buffer, else null.
static void *mapped_host(void *h)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int hpxfft_execute_r2c_host(hpxfft_plan p, void *h)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (!h) return fail(HPXFFT_ERR_INVALID_ARG, "null host buffer");
    int rc = ensure_dbuf(p);
    if (rc) return rc;
    const size_t bytes = p->nx * p->ncol * p->real_bytes * p->batch;
    cudaError_t e;
    if ((rc = collect(*p)) != HPXFFT_OK) return rc;
    if ((e = cudaEventRecord(p->ev_copy[0], p->stream)) != cudaSuccess) return cuda_fail(e, "event");
    // page-locked memory read and written in place by the kernels, except by
    // the paths of dimensions outside the direct kernels' sizes
    const bool alt = p->alt_row.on || p->alt_col.on;
    void *hd = ((uintptr_t)h & 15) || alt ? nullptr : mapped_host(h);
    const bool pipelined = hd && pipelined_shape(*p);
    if (pipelined) {
        // page-locked memory, two-step column plan: chunked copies overlapped
        // with the kernels
        if ((e = ensure_pipeline(*p)) != cudaSuccess) return cuda_fail(e, "copy streams");
        if ((e = dispatch_forward_pipelined(*p, h)) != cudaSuccess) return cuda_fail(e, "pipelined forward");
    } else if (hd) {
        // page-locked host memory: the row pass reads it and the last column
        // step writes it over the host link, no staging copies
        if ((e = dispatch_forward(*p, hd, p->dbuf, hd, 0)) != cudaSuccess) return cuda_fail(e, "forward launch");
        if (!p->col_two_step &&
            (e = cudaMemcpyAsync(h, p->dbuf, bytes, cudaMemcpyDeviceToHost, p->stream)) != cudaSuccess)
            return cuda_fail(e, "device to host copy");
    } else {
        if ((e = cudaMemcpyAsync(p->dbuf, h, bytes, cudaMemcpyHostToDevice, p->stream)) != cudaSuccess)
            return cuda_fail(e, "host to device copy");
        if ((e = dispatch_forward(*p, p->dbuf, p->dbuf)) != cudaSuccess) return cuda_fail(e, "forward launch");
        if ((e = cudaMemcpyAsync(h, p->dbuf, bytes, cudaMemcpyDeviceToHost, p->stream)) != cudaSuccess)
            return cuda_fail(e, "device to host copy");
    }
    if ((e = cudaEventRecord(p->ev_copy[1], p->stream)) != cudaSuccess) return cuda_fail(e, "event");
    if ((e = cudaEventSynchronize(p->ev_copy[1])) != cudaSuccess) return cuda_fail(e, "transform");
    p->pending_copy = true;
    p->last_zero_copy = hd != nullptr && !pipelined;
    p->last_pipelined = pipelined;
    if ((rc = collect(*p)) != HPXFFT_OK) return rc;
    p->meas["host_pipelined"] = pipelined ? 1.0 : 0.0;
    if (pipelined) {
        // h2d: until the last input chunk landed; d2h: from the last column
        // step to the last output byte (the rest of both overlaps the kernels)
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, p->ev_copy[0], p->chunk_in[hpxfft_plan_s::kChunks - 1]);
        cudaEventElapsedTime(&b, p->kev[(p->next - 1) % hpxfft_plan_s::kSlots][2], p->ev_copy[1]);
        p->meas["h2d"] = 1e-3 * a;
        p->meas["d2h"] = 1e-3 * b;
    }
    return check_device_error(p);
}

int hpxfft_plan_synchronize(hpxfft_plan p)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    cudaError_t e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "transform");
    return check_device_error(p);
}

int hpxfft_execute_c2r(hpxfft_plan p, void *d)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (!d) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    cudaError_t e = dispatch_inverse(*p, d, 0);
    if (e != cudaSuccess) return cuda_fail(e, "inverse launch");
    return HPXFFT_OK;
}

int hpxfft_execute_r2c_backward(hpxfft_plan p, void *d)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (!d) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    cudaError_t e = dispatch_inverse(*p, d, 1);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
    return HPXFFT_OK;
}

int hpxfft_execute_r2c_backward_host(hpxfft_plan p, void *h)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    if (!h) return fail(HPXFFT_ERR_INVALID_ARG, "null host buffer");
    int rc = ensure_dbuf(p);
    if (rc) return rc;
    const size_t bytes = p->nx * p->ncol * p->real_bytes * p->batch;
    cudaError_t e;
    if ((rc = collect(*p)) != HPXFFT_OK) return rc;
    if ((e = cudaMemcpyAsync(p->dbuf, h, bytes, cudaMemcpyHostToDevice, p->stream)) != cudaSuccess)
        return cuda_fail(e, "host to device copy");
    if ((e = dispatch_inverse(*p, p->dbuf, 1)) != cudaSuccess) return cuda_fail(e, "adjoint launch");
    if ((e = cudaMemcpyAsync(h, p->dbuf, bytes, cudaMemcpyDeviceToHost, p->stream)) != cudaSuccess)
        return cuda_fail(e, "device to host copy");
    if ((e = cudaStreamSynchronize(p->stream)) != cudaSuccess) return cuda_fail(e, "adjoint");
    if ((rc = collect(*p)) != HPXFFT_OK) return rc;
    return check_device_error(p);
}

int hpxfft_get_measurement(hpxfft_plan p, const char *name, double *value)
{
    if (!p || !name || !value) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    int rc = collect(*p);
    if (rc) return rc;
    auto it = p->meas.find(name);
    *value = it == p->meas.end() ? 0.0 : it->second;
    return HPXFFT_OK;
}

int hpxfft_timing_stats(hpxfft_plan p, double *first_mean, double *second_mean, double *total_mean,
                        long long *count)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    int rc = collect(*p);
    if (rc) return rc;
    const double n = p->nsum ? (double)p->nsum : 1.0;
    p->meas["mean_first"] = p->sum_first / n;
    p->meas["mean_second"] = p->sum_second / n;
    // with the two-step column pass: time from the row kernel's start to the
    // end of step A, so step A alone = that minus the row kernel
    p->meas["mean_col_step_a"] = p->col_two_step ? p->sum_step_a / n - p->sum_first / n : 0.0;
    p->meas["mean_col_step_b"] = p->col_two_step ? p->sum_second / n - p->meas["mean_col_step_a"] : 0.0;
    p->meas["column_steps"] = p->col_two_step ? 2.0 : 1.0;
    if (first_mean) *first_mean = p->sum_first / n;
    if (second_mean) *second_mean = p->sum_second / n;
    if (total_mean) *total_mean = p->sum_total / n;
    if (count) *count = p->nsum;
    return HPXFFT_OK;
}

int hpxfft_timing_reset(hpxfft_plan p)
{
    if (!p) return fail(HPXFFT_ERR_STATE, "null plan");
    int rc = collect(*p);
    p->sum_first = p->sum_second = p->sum_total = p->sum_step_a = 0.0;
    p->nsum = 0;
    return rc;
}

int hpxfft_write_plan(hpxfft_plan p, const char *path)
{
    if (!p || !path) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    FILE *f = fopen(path, "a");
    if (!f) return fail(HPXFFT_ERR_IO, std::string("Failed to open file: ") + path);
    auto columns_of = [](const hpxfft_plan_s &q, const char *what) {
        if (!q.col_two_step) return describe(q, q.col, what, q.nx);
        return describe(q, q.colA, "c2c-stepA", (size_t)q.N2) + "\n" + describe(q, q.colB, "c2c-stepB", (size_t)q.N1);
    };
    if (p->alt_row.on && p->alt_row.bluestein)
        fprintf(f, "GPU r2c 1D plan (rows transposed into columns; Bluestein, length %zu through %zu):\n%s\n", p->ny / 2,
                p->alt_row.M, columns_of(*p->alt_row.sub, "c2c").c_str());
    else if (p->alt_row.on)
        fprintf(f, "GPU r2c 1D plan (rows transposed into columns, length %zu):\n%s\n", p->ny / 2,
                columns_of(*p->alt_row.sub, "c2c").c_str());
    else
        fprintf(f, "GPU r2c 1D plan:\n%s\n", describe(*p, p->row, "r2c", p->ny).c_str());
    if (p->alt_col.on) {
        fprintf(f, "GPU c2c 1D plan (Bluestein, length %zu through %zu):\n%s\n\n", p->nx, p->alt_col.M,
                columns_of(*p->alt_col.sub, "c2c").c_str());
    } else if (p->col_two_step) {
        fprintf(f, "GPU c2c 1D plan (four-step, %d x %d%s):\n%s\n%s\n\n", p->N1, p->N2,
                p->ff_pairs ? ", float-float pairs between kernels" : "",
                describe(*p, p->colA, "c2c-stepA", (size_t)p->N2).c_str(),
                describe(*p, p->colB, "c2c-stepB", (size_t)p->N1).c_str());
    } else {
        fprintf(f, "GPU c2c 1D plan:\n%s\n\n", describe(*p, p->col, "c2c", p->nx).c_str());
    }
    // how the plan's choices were made: fixed rules ("estimate"), a timed
    // search over the candidates, or a cached (wisdom) choice
    fprintf(f, "GPU plan choice (flag %s, from %s): %s\n", p->flag.c_str(), p->tuned_from.c_str(),
            describe_choice(p->choice).c_str());
    for (auto &c : p->tuning)
        fprintf(f, "  candidate %s: %.4f ms%s\n", c.first.c_str(), c.second,
                c.first == describe_choice(p->choice) ? " (chosen)" : "");
    fprintf(f, "\n");
    fclose(f);
    return HPXFFT_OK;
}

int hpxfft_host_alloc(void **ptr, size_t bytes)
{
    if (!ptr) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    if (cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(HPXFFT_ERR_ALLOC, "pinned host allocation");
    }
    return HPXFFT_OK;
}

int hpxfft_host_free(void *ptr)
{
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) return fail(HPXFFT_ERR_CUDA, "cudaFreeHost");
    return HPXFFT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free forward transform (hpxfft_execute_r2c_noalloc).
//
// The plan API allocates device memory (twiddle tables) when a plan is
// created.  Some callers cannot do that: an application whose own pool
// allocator has reserved all device memory up front (a cudaMalloc then fails
// or fragments the pool), or a latency-critical pipeline that must not issue
// cudaMalloc / cudaFree because they can synchronise the whole device.  This
// entry point serves them: the FP64 transform with the same kernels, its
// twiddle tables written into one file-scope __device__ array that every GPU
// loading the library holds until the process exits.
// ---------------------------------------------------------------------------
namespace hpxfft_gpu {

constexpr size_t kNoAllocMaxLen = 16384;                  // largest n_row and largest ny
constexpr size_t kNoAllocScratchBytes = (size_t)1 << 20;  // 1 MiB: 4 tables of <= 16384 pairs
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mutex;
static void *g_noalloc_ptr[kMaxDevices];  // device address of g_noalloc_scratch, per device

// The plan's own row and column rules (plan_rows and plan_cols use no heap).
// The columns always take the single-kernel cluster pass: the two-kernel
// four-step pass a plan picks for power-of-two n_row >= 8192 needs a scratch
// array as large as the data, which this entry point cannot allocate.
static bool noalloc_shape(hpxfft_plan_s &p) { return plan_rows(p) && plan_cols(p); }

// Per-pass tables of a compile-time chain written at `dst` (no allocation).
static cudaError_t noalloc_fixed_tables(DimPlan &d, bool rows, unsigned char *dst, size_t cap, size_t &used,
                                        cudaStream_t st)
{
    d.FL = 0;
    used = 0;
    if (!(rows ? RowLaunch<ArithFF>::has_fixed(d.L, d.log2W, d.C) : ColLaunch<ArithFF>::has_fixed(d.L, d.log2W, d.C)))
        return cudaSuccess;
    size_t off = 0;
    for (int Ls = 1; Ls < d.L;) {
        const int R = fixed_radix(d.L, Ls, ArithFF::kEPTFixed);
        if (Ls > 1) {
            if ((off + (size_t)Ls * (R - 1)) * 16 > cap) return cudaErrorInvalidValue;
            cudaError_t e = TwiddleLaunch<ArithFF>::pass(dst + off * 16, Ls, R, st);
            if (e != cudaSuccess) return e;
            off += (size_t)Ls * (R - 1);
        }
        Ls *= R;
    }
    d.ptab = dst;
    d.FL = d.L;
    d.shape.threads = fixed_threads(d.L, d.log2W, ArithFF::kEPTFixed);
    used = (off * 16 + 255) & ~(size_t)255;
    return cudaSuccess;
}

}  // namespace hpxfft_gpu

extern "C" int hpxfft_execute_r2c_noalloc(const void *d_in, void *d_out, size_t n_row, size_t n_col, void *stream)
{
    using namespace hpxfft_gpu;
    if (!d_in || !d_out) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    if (((uintptr_t)d_in | (uintptr_t)d_out) & 15) return fail(HPXFFT_ERR_INVALID_ARG, "buffers must be 16-byte aligned");
    if (n_row == 0) return fail(HPXFFT_ERR_INVALID_ARG, "empty array");
    if (n_col < 4 || n_col % 2) return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "n_col must be 2*(ny/2+1) with ny >= 2 even");
    if (n_row > kNoAllocMaxLen || n_col - 2 > kNoAllocMaxLen)
        return fail(HPXFFT_ERR_UNSUPPORTED_SIZE,
                    "hpxfft_execute_r2c_noalloc handles n_row <= 16384 and ny <= 16384 (its 1 MiB static scratch); "
                    "use a plan for larger arrays");
    hpxfft_plan_s p;
    p.nx = n_row;
    p.dcy = n_col / 2;
    p.ny = 2 * p.dcy - 2;
    p.M = p.ny / 2;
    p.ncol = n_col;
    p.batch = 1;
    p.prec = HPXFFT_PREC_F64;
    p.real_bytes = 8;
    p.tw_elem = 16;
    if (!noalloc_shape(p))
        return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "sizes must have no prime factor above 13");

    // one-time set-up per device, with that device current: the device
    // address of the static scratch array and the kernel attributes
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(HPXFFT_ERR_CUDA, "device index out of range");
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
            g_noalloc_ptr[dev] = ptr;
        }
        base = static_cast<unsigned char *>(g_noalloc_ptr[dev]);
    }
    if ((e = prepare_once<ArithFF>()) != cudaSuccess) return cuda_fail(e, "kernel attributes");

    // carve the scratch: full row table (2M pairs), full column table (nx
    // pairs), then the per-pass tables; every table is rewritten by this call
    cudaStream_t st = (cudaStream_t)stream;
    size_t off = 0;
    p.tw_row = base + off;
    off += ((2 * p.M * 16) + 255) & ~(size_t)255;
    p.tw_col = base + off;
    off += ((p.nx * 16) + 255) & ~(size_t)255;
    size_t used = 0;
    if ((e = noalloc_fixed_tables(p.row, true, base + off, kNoAllocScratchBytes - off, used, st)) != cudaSuccess)
        return cuda_fail(e, "row twiddles");
    off += used;
    if ((e = noalloc_fixed_tables(p.col, false, base + off, kNoAllocScratchBytes - off, used, st)) != cudaSuccess)
        return cuda_fail(e, "column twiddles");
    off += used;
    if (off > kNoAllocScratchBytes) return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "scratch too small");
    if ((e = TwiddleLaunch<ArithFF>::full(p.tw_row, (int)(2 * p.M), st)) != cudaSuccess ||
        (e = TwiddleLaunch<ArithFF>::full(p.tw_col, (int)p.nx, st)) != cudaSuccess)
        return cuda_fail(e, "twiddle generation");
    if ((e = RowLaunch<ArithFF>::r2c(row_args(p, d_in, d_out, 0), p.row.shape, p.row.FL, st)) != cudaSuccess)
        return cuda_fail(e, "row kernel");
    if ((e = ColLaunch<ArithFF>::run(col_args(p, d_out), -1, p.col.shape, p.col.FL, st)) != cudaSuccess)
        return cuda_fail(e, "column kernel");
    return HPXFFT_OK;
}

// ---------------------------------------------------------------------------
// Slab decomposition over P ranks (hpxfft_slab_*): the per-locality compute of
// hpxfft::distributed::loop::fft_2d_r2c (core/src/distributed/loop.cpp:130-272)
// with index maps that are correct for any P.  Rank r holds global rows
// r * n_x_local + x of the padded input.  dcy = n_col / 2 complex columns are
// split into P tiles of w = ceil(dcy / P) columns (the last tile padded with
// zeros), so dcy need not be a multiple of P.
//   rows:    row r2c of the local slab, then pack: send[d][x][k] = X[x][d w + k]
//   (caller: all_to_all, tile d to rank d)
//   columns: recv[s][x][k] is global row s n_x_local + x of my w columns, so
//            recv is the column slab [nx][w]; column c2c in place; tile d of
//            the result holds the rows kx of rank d: ready to send back
//   (caller: all_to_all, tile d to rank d)
//   finish:  out[x][s w + k] = recv2[s][x][k] for s w + k < dcy
// The reference's transposes interleave the slabs cyclically, which is only
// right for P = 1 (core/src/distributed/loop.cpp:87-127); its pack and
// exchange steps are core/src/distributed/loop.cpp:19-84.
// ---------------------------------------------------------------------------
namespace hpxfft_gpu {

template <class C>
__global__ void slab_pack_kernel(const C *__restrict__ rows, C *__restrict__ send, int n_x_local, int dcy, int w)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x, d = blockIdx.z;
    if (k >= w) return;
    const int col = d * w + k;
    for (int x = blockIdx.y; x < n_x_local; x += gridDim.y) {
        C v{};
        if (col < dcy) v = rows[(long long)x * dcy + col];
        send[((long long)d * n_x_local + x) * w + k] = v;
    }
}

template <class C>
__global__ void slab_unpack_kernel(const C *__restrict__ recv, C *__restrict__ rows, int n_x_local, int dcy, int w)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= dcy) return;
    const int s = col / w, k = col - s * w;
    for (int x = blockIdx.y; x < n_x_local; x += gridDim.y)
        rows[(long long)x * dcy + col] = recv[((long long)s * n_x_local + x) * w + k];
}

}  // namespace hpxfft_gpu

struct hpxfft_slab_s {
    hpxfft_plan rows = nullptr, cols = nullptr;
    size_t nxl = 0, nx = 0, ncol = 0, dcy = 0, P = 1, rank = 0, w = 0, elem = 16;
    int prec = HPXFFT_PREC_F64;
    cudaEvent_t ev[8] = {};
    bool ran_rows = false, ran_cols = false, ran_finish = false;
    std::map<std::string, double> meas;
};

namespace hpxfft_gpu {

static cudaError_t slab_pack(hpxfft_slab_s &s, const void *rows, void *send, cudaStream_t st)
{
    const unsigned gy = (unsigned)std::min<size_t>(s.nxl, 65535);
    dim3 grid((unsigned)((s.w + 255) / 256), gy, (unsigned)s.P);
    if (s.elem == 16)
        slab_pack_kernel<double2><<<grid, 256, 0, st>>>((const double2 *)rows, (double2 *)send, (int)s.nxl,
                                                         (int)s.dcy, (int)s.w);
    else
        slab_pack_kernel<float2><<<grid, 256, 0, st>>>((const float2 *)rows, (float2 *)send, (int)s.nxl, (int)s.dcy,
                                                        (int)s.w);
    return cudaGetLastError();
}

static cudaError_t slab_unpack(hpxfft_slab_s &s, const void *recv, void *rows, cudaStream_t st)
{
    const unsigned gy = (unsigned)std::min<size_t>(s.nxl, 65535);
    dim3 grid((unsigned)((s.dcy + 255) / 256), gy, 1);
    if (s.elem == 16)
        slab_unpack_kernel<double2><<<grid, 256, 0, st>>>((const double2 *)recv, (double2 *)rows, (int)s.nxl,
                                                           (int)s.dcy, (int)s.w);
    else
        slab_unpack_kernel<float2><<<grid, 256, 0, st>>>((const float2 *)recv, (float2 *)rows, (int)s.nxl,
                                                          (int)s.dcy, (int)s.w);
    return cudaGetLastError();
}

static double event_s(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();
        return 0.0;
    }
    return 1e-3 * ms;
}

}  // namespace hpxfft_gpu

extern "C" {

int hpxfft_slab_create(hpxfft_slab *out, size_t n_row_local, size_t n_col, size_t n_ranks, size_t rank, int precision,
                       const char *plan_flag)
{
    if (!out) return fail(HPXFFT_ERR_INVALID_ARG, "slab pointer is null");
    *out = nullptr;
    if (!valid_flag(plan_flag)) return fail(HPXFFT_ERR_INVALID_ARG, "Invalid FFTW plan flag string");
    if (n_ranks == 0 || rank >= n_ranks) return fail(HPXFFT_ERR_INVALID_ARG, "rank must be below n_ranks");
    if (n_row_local == 0) return fail(HPXFFT_ERR_INVALID_ARG, "empty slab");
    if (n_col < 4 || n_col % 2) return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "n_col must be 2*(ny/2+1) with ny >= 2 even");
    if (n_ranks > 65535 || n_row_local * n_ranks > (1u << 30))
        return fail(HPXFFT_ERR_UNSUPPORTED_SIZE, "dimension too large");
    hpxfft_slab_s *s = new (std::nothrow) hpxfft_slab_s();
    if (!s) return fail(HPXFFT_ERR_ALLOC, "host allocation failed");
    s->nxl = n_row_local;
    s->P = n_ranks;
    s->rank = rank;
    s->nx = n_row_local * n_ranks;
    s->ncol = n_col;
    s->dcy = n_col / 2;
    s->w = (s->dcy + n_ranks - 1) / n_ranks;
    s->prec = precision;
    s->elem = f32_storage(precision) ? 8 : 16;
    int rc = create_plan(&s->rows, n_row_local, n_col, 1, precision, plan_flag, kPlanRows);
    if (rc == HPXFFT_OK) rc = create_plan(&s->cols, s->nx, 2 * s->w, 1, precision, plan_flag, kPlanColumns);
    for (auto &ev : s->ev)
        if (rc == HPXFFT_OK && cudaEventCreate(&ev) != cudaSuccess) rc = fail(HPXFFT_ERR_CUDA, "event");
    if (rc != HPXFFT_OK) {
        std::string msg = g_last_error;
        hpxfft_slab_destroy(s);
        return fail(rc, msg);
    }
    s->cols->stream = s->rows->stream;  // one stream orders every phase
    s->meas["plan"] = s->rows->meas["plan"] + s->cols->meas["plan"];
    *out = s;
    return HPXFFT_OK;
}

int hpxfft_slab_destroy(hpxfft_slab s)
{
    if (!s) return fail(HPXFFT_ERR_STATE, "null slab");
    if (s->cols) {
        if (s->rows) s->cols->stream = s->cols->own_stream;
        hpxfft_plan_destroy(s->cols);
    }
    if (s->rows) hpxfft_plan_destroy(s->rows);
    for (auto &ev : s->ev)
        if (ev) cudaEventDestroy(ev);
    delete s;
    return HPXFFT_OK;
}

int hpxfft_slab_set_stream(hpxfft_slab s, void *stream)
{
    if (!s) return fail(HPXFFT_ERR_STATE, "null slab");
    s->rows->stream = (cudaStream_t)stream;
    s->cols->stream = (cudaStream_t)stream;
    return HPXFFT_OK;
}

int hpxfft_slab_tile_bytes(hpxfft_slab s, size_t *bytes)
{
    if (!s || !bytes) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    *bytes = s->nxl * s->w * s->elem;
    return HPXFFT_OK;
}

int hpxfft_slab_rows(hpxfft_slab s, void *d_values, void *d_send)
{
    if (!s) return fail(HPXFFT_ERR_STATE, "null slab");
    if (!d_values || !d_send) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    if (((uintptr_t)d_values | (uintptr_t)d_send) & 15) return fail(HPXFFT_ERR_INVALID_ARG, "buffers must be 16-byte aligned");
    cudaStream_t st = s->rows->stream;
    cudaError_t e = cudaEventRecord(s->ev[0], st);
    if (e == cudaSuccess) e = dispatch_rows_only(*s->rows, d_values, d_values);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[1], st);
    if (e == cudaSuccess) e = slab_pack(*s, d_values, d_send, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[2], st);
    if (e != cudaSuccess) return cuda_fail(e, "slab rows");
    s->ran_rows = true;
    return HPXFFT_OK;
}

int hpxfft_slab_columns(hpxfft_slab s, void *d_recv)
{
    if (!s) return fail(HPXFFT_ERR_STATE, "null slab");
    if (!d_recv) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    if ((uintptr_t)d_recv & 15) return fail(HPXFFT_ERR_INVALID_ARG, "buffers must be 16-byte aligned");
    cudaStream_t st = s->cols->stream;
    cudaError_t e = cudaEventRecord(s->ev[3], st);
    if (e == cudaSuccess) e = dispatch_columns_only(*s->cols, d_recv);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[4], st);
    if (e != cudaSuccess) return cuda_fail(e, "slab columns");
    s->ran_cols = true;
    return HPXFFT_OK;
}

int hpxfft_slab_finish(hpxfft_slab s, const void *d_recv, void *d_values)
{
    if (!s) return fail(HPXFFT_ERR_STATE, "null slab");
    if (!d_recv || !d_values) return fail(HPXFFT_ERR_INVALID_ARG, "null device buffer");
    if (((uintptr_t)d_recv | (uintptr_t)d_values) & 15) return fail(HPXFFT_ERR_INVALID_ARG, "buffers must be 16-byte aligned");
    cudaStream_t st = s->rows->stream;
    cudaError_t e = cudaEventRecord(s->ev[5], st);
    if (e == cudaSuccess) e = slab_unpack(*s, d_recv, d_values, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[6], st);
    if (e != cudaSuccess) return cuda_fail(e, "slab finish");
    s->ran_finish = true;
    return HPXFFT_OK;
}

int hpxfft_slab_synchronize(hpxfft_slab s)
{
    if (!s) return fail(HPXFFT_ERR_STATE, "null slab");
    cudaError_t e = cudaStreamSynchronize(s->rows->stream);
    if (e != cudaSuccess) return cuda_fail(e, "slab");
    int rc = check_device_error(s->rows);
    return rc == HPXFFT_OK ? check_device_error(s->cols) : rc;
}

// Device seconds of the local phases of the last run, with the reference's
// keys (core/src/distributed/loop.cpp:260-268); the exchanges are the
// caller's, so first_comm and second_comm are not measured here.
int hpxfft_slab_get_measurement(hpxfft_slab s, const char *name, double *value)
{
    if (!s || !name || !value) return fail(HPXFFT_ERR_INVALID_ARG, "null argument");
    int rc = hpxfft_slab_synchronize(s);
    if (rc != HPXFFT_OK) return rc;
    collect(*s->rows);
    collect(*s->cols);
    if (s->ran_rows) {
        s->meas["first_fftw"] = event_s(s->ev[0], s->ev[1]);
        s->meas["first_split"] = event_s(s->ev[1], s->ev[2]);
    }
    s->meas["first_trans"] = 0.0;  // the received tiles are the column slab
    if (s->ran_cols) s->meas["second_fftw"] = event_s(s->ev[3], s->ev[4]);
    s->meas["second_split"] = 0.0;  // the column slab is the send layout
    if (s->ran_finish) s->meas["second_trans"] = event_s(s->ev[5], s->ev[6]);
    s->meas["n_ranks"] = (double)s->P;
    s->meas["rank"] = (double)s->rank;
    s->meas["tile_columns"] = (double)s->w;
    auto it = s->meas.find(name);
    *value = it == s->meas.end() ? 0.0 : it->second;
    return HPXFFT_OK;
}

}  // extern "C"
