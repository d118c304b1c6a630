// Many 2D r2c transforms of different sizes in one persistent launch.
//
// The host flattens a batch into work items: row items (one CTA-sized group
// of rows of one instance) and column items (one strip of columns of one
// instance).  Persistent CTAs take items in order from an atomic counter.  A
// column item may start only when every row item of its instance has
// finished: the row item's CTA publishes its completion with a release
// increment of the instance's counter, the column item's first thread polls
// it (a bounded wait that reports HPXFFT_ERR_TIMEOUT instead of hanging).
// Items are only ever held by running CTAs, and every row item of an
// instance is queued before its column items, so the waits always end.
//
// Rows of instance i are queued `lag` instances ahead of its columns, so an
// instance's data is still in L2 when its column items read it back.
#pragma once
#include "fft_kernels.cuh"

namespace hpxfft_gpu {

struct BatchDim {
    PassPlan pp;
    int L;
    int log2W;
    int fixed_id;    // index into the compile-time list below, -1: runtime plan
    int ptab;        // complex entries into the twiddle pool (per-pass tables)
};

// Compile-time (L, log2 interleave) shapes of the FP32 batch kernel: the
// lengths 2^k, 3*2^k, 5*2^k between 128 and 4096, each packed to fill a CTA of
// at most 8192 elements (rows: L = ny/2, columns: L = nx).
#define HPXFFT_BATCH_ROWS_F32(X) \
    X(0, 128, 6) X(1, 192, 5) X(2, 256, 5) X(3, 320, 4) X(4, 384, 4) X(5, 512, 4) X(6, 768, 3) X(7, 1024, 3) \
    X(8, 1280, 2) X(9, 1536, 2) X(10, 2048, 2)
#define HPXFFT_BATCH_COLS_F32(X) \
    X(0, 256, 5) X(1, 384, 4) X(2, 512, 4) X(3, 640, 3) X(4, 768, 3) X(5, 1024, 3) X(6, 1536, 2) X(7, 2048, 2) \
    X(8, 2560, 1) X(9, 3072, 1) X(10, 4096, 1)

struct BatchInst {
    long long offset;  // reals from the arena base
    int nx, M, dcy, ncol;
    int row_dim, col_dim;
    int row_items;
    int tw_row, tw_col;  // complex entries into the twiddle pool
};

struct BatchItem {
    int inst;
    int kind;  // 0 row group, 1 column strip
    int group;
    int pad;
};

struct BatchArgs {
    void *arena;
    const BatchInst *insts;
    const BatchItem *items;
    const BatchDim *dims;
    const void *twpool;
    int nitems;
    int *counters;  // [0] next item, [1] timeout flag, [2 + i] row items done of instance i
    long long spin_limit;
};

constexpr int kBatchThreads = 512;

// One body per compiled shape, not inlined: each gets its own register
// allocation instead of the union of all of them in the persistent loop.
template <class A, int FL, int FW>
__device__ __noinline__ void batch_row(const RowArgs &a, int group)
{
    row_r2c_body<A, 1, FL, FW>(a, group, 0);
}
template <class A, int FL, int FW>
__device__ __noinline__ void batch_col(const ColArgs &a, int group)
{
    col_body<A, 1, -1, FL, FW>(a, group, 0);
}

// Two CTAs per SM (64 registers, <= 70 KB shared memory each): while one
// streams an item in or out, the other computes.  Thread 0 takes the item,
// does the bounded wait of a column item and builds the body's arguments in
// shared memory: one copy per CTA, which the non-inlined bodies read
// through a reference, instead of one per thread on the thread's stack
// (local memory, whose traffic to L2 and DRAM outweighed the data's).
template <class A>
__global__ void __launch_bounds__(kBatchThreads, 2) batch_kernel(BatchArgs b)
{
    using T = typename A::T;
    using S = typename A::S;
    __shared__ int s_item, s_ok, s_kind, s_group, s_fixed;
    __shared__ RowArgs s_ra;
    __shared__ ColArgs s_ca;
    int *next = b.counters, *timeout = b.counters + 1, *rows_done = b.counters + 2;
    for (;;) {
        if (threadIdx.x == 0) {
            const int it = atomicAdd(next, 1);
            s_item = it;
            if (it < b.nitems) {
                const BatchItem item = b.items[it];
                const BatchInst in = b.insts[item.inst];
                S *base = reinterpret_cast<S *>(b.arena) + in.offset;
                const cpx<T> *pool = reinterpret_cast<const cpx<T> *>(b.twpool);
                s_kind = item.kind;
                s_group = item.group;
                s_ok = 1;
                if (item.kind == 0) {
                    const BatchDim &d = b.dims[in.row_dim];
                    RowArgs ra{};
                    ra.in = base;
                    ra.out = base;
                    ra.in_stride = ra.out_stride = in.ncol;
                    ra.nrows = in.nx;
                    ra.M = in.M;
                    ra.log2W = d.log2W;
                    ra.pp = d.pp;
                    ra.tw = pool + in.tw_row;
                    ra.Ltab = 2 * in.M;
                    ra.ptab = pool + d.ptab;
                    s_ra = ra;
                    s_fixed = d.fixed_id;
                } else {
                    long long spins = 0;
                    while (atomicAdd(&rows_done[item.inst], 0) < in.row_items) {
                        if (++spins > b.spin_limit) {
                            s_ok = 0;
                            atomicExch(timeout, 1);
                            break;
                        }
                        __nanosleep(128);
                    }
                    __threadfence();
                    const BatchDim &d = b.dims[in.col_dim];
                    ColArgs ca{};
                    ca.data = base;
                    ca.row_stride = in.ncol;
                    ca.nx = in.nx;
                    ca.ncols = in.dcy;
                    ca.log2W = d.log2W;
                    ca.pp = d.pp;
                    ca.tw = pool + in.tw_col;
                    ca.Ltab = in.nx;
                    ca.ptab = pool + d.ptab;
                    s_ca = ca;
                    s_fixed = d.fixed_id;
                }
            }
        }
        __syncthreads();
        const int it = s_item;
        if (it >= b.nitems) return;
        const int group = s_group, fixed = s_fixed;
        if (s_kind == 0) {
            bool done = false;
            if constexpr (sizeof(S) == 4) {
                switch (fixed) {
#define HPXFFT_X(ID, L_, W_)                                \
    case ID:                                                \
        batch_row<A, L_, W_>(s_ra, group);                  \
        done = true;                                        \
        break;
                    HPXFFT_BATCH_ROWS_F32(HPXFFT_X)
#undef HPXFFT_X
                default: break;
                }
            }
            if (!done) batch_row<A, 0, 0>(s_ra, group);
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) atomicAdd(&rows_done[b.items[it].inst], 1);
        } else if (s_ok) {
            bool done = false;
            if constexpr (sizeof(S) == 4) {
                switch (fixed) {
#define HPXFFT_X(ID, L_, W_)                                  \
    case ID:                                                  \
        batch_col<A, L_, W_>(s_ca, group);                    \
        done = true;                                          \
        break;
                    HPXFFT_BATCH_COLS_F32(HPXFFT_X)
#undef HPXFFT_X
                default: break;
                }
            }
            if (!done) batch_col<A, 0, 0>(s_ca, group);
        }
        __syncthreads();  // the shared arguments are rewritten next iteration
    }
}

}  // namespace hpxfft_gpu
