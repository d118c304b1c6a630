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
};

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

template <class A>
__global__ void __launch_bounds__(kBatchThreads, 1) batch_kernel(BatchArgs b)
{
    using T = typename A::T;
    using S = typename A::S;
    __shared__ int s_item, s_ok;
    int *next = b.counters, *timeout = b.counters + 1, *rows_done = b.counters + 2;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= b.nitems) return;
        const BatchItem item = b.items[it];
        const BatchInst in = b.insts[item.inst];
        S *base = reinterpret_cast<S *>(b.arena) + in.offset;
        const cpx<T> *pool = reinterpret_cast<const cpx<T> *>(b.twpool);
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
            row_r2c_body<A, 1, 0, 0>(ra, item.group, 0);
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) atomicAdd(&rows_done[item.inst], 1);
        } else {
            if (threadIdx.x == 0) {
                int ok = 1;
                long long spins = 0;
                while (atomicAdd(&rows_done[item.inst], 0) < in.row_items) {
                    if (++spins > b.spin_limit) {
                        ok = 0;
                        atomicExch(timeout, 1);
                        break;
                    }
                    __nanosleep(128);
                }
                __threadfence();
                s_ok = ok;
            }
            __syncthreads();
            if (s_ok) {
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
                col_body<A, 1, -1, 0, 0>(ca, item.group, 0);
            }
        }
        __syncthreads();  // s_item is rewritten next iteration
    }
}

}  // namespace hpxfft_gpu
