// Replay items and span-state access shared by the item pipeline kernels.
#pragma once

#include "tsg_query.cuh"

namespace tsg {

// One replay item: a node whose counts or parent changed across one
// transition (or, at the first tree, a node alive there), with its counts
// before (x0) and after (x1) and its parent before (p0) and after (p1), as
// local ids of the span whose replay wrote the item (-1: no parent).  Its
// value is F(x1) * bl1 - F(x0) * bl0 with bl = time[parent] - time[u]
// (0 without a parent).
template <int KQ>
struct __align__(16) Item {
    uint64_t x0[KQ];
    uint64_t x1[KQ];
    int32_t u, p0, p1, pad;
};

template <int KQ>
__device__ __forceinline__ Pack item_pack(const uint64_t *a)
{
    Pack p;
    p.lo = a[0];
    p.hi = KQ > 1 ? a[KQ > 1 ? 1 : 0] : 0ull;
    return p;
}

template <int KQ>
__device__ __forceinline__ void item_put(Item<KQ> *it, const Pack &x0, const Pack &x1, int32_t u,
    int32_t p0, int32_t p1)
{
    Item<KQ> v;
    v.x0[0] = x0.lo;
    v.x1[0] = x1.lo;
    if (KQ > 1) {
        v.x0[KQ > 1 ? 1 : 0] = x0.hi;
        v.x1[KQ > 1 ? 1 : 0] = x1.hi;
    }
    v.u = u;
    v.p0 = p0;
    v.p1 = p1;
    v.pad = 0;
    *it = v;
}

// Asynchronous global -> shared copies (cp.async, sm_80 and later): the
// item replay stages each tree's inputs a few trees ahead of use.
__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// events and mutations of a tree staged in shared memory ahead of the
// replay (a tree's further ones are read from global memory when used):
// trees have about eight edge events and a few mutations, and the ring's
// bytes bound how many compact replays an SM holds at once
#define TSG_STAGE_N 16

// One tree's replay inputs, staged in shared memory ahead of use: the edge
// events into the tree, its mutations, its item range, and the first
// TSG_STAGE_N event encodings, mutation encodings and leaf sample-set masks
// of each.
struct __align__(16) ReplayStage {
    int4 ev;           // removal offset, removals, insertion offset, insertions
    int2 mr;           // mutations [first, end)
    int64_t ioff[2];   // items [first, end)
    int2 pc[TSG_STAGE_N];       // event (parent, child) encodings
    uint32_t cm[TSG_STAGE_N];   // leaf child masks
    int32_t menc[TSG_STAGE_N];  // mutation node encodings
    uint32_t mmask[TSG_STAGE_N];  // leaf mutation node masks
};

// an entry of the replay's open touch list (shared memory)
template <int KQ>
struct TouchEntry {
    uint64_t x0[KQ];
    uint32_t u;
    int32_t p0;
};

// branch lengths of an item from its span's node times
template <int KQ>
__device__ __forceinline__ void item_branches(const Item<KQ> &it, const double *time, double &bl0,
    double &bl1)
{
    const double tu = time[it.u];
    bl0 = it.p0 >= 0 ? time[it.p0] - tu : 0.0;
    bl1 = it.p1 >= 0 ? time[it.p1] - tu : 0.0;
}

// loads of span state that atomics also update: shared memory is coherent;
// in global memory they must bypass L1
template <typename IdxT>
__device__ __forceinline__ uint64_t st_ld(const uint64_t *p)
{
    if (sizeof(IdxT) == 2) {
        return *p;
    }
    return __ldcg((const unsigned long long *) p);
}

// seek counters are in global memory and updated by atomics
template <typename IdxT>
__device__ __forceinline__ uint32_t st_ld32(const uint32_t *p)
{
    return __ldcg(p);
}

template <typename IdxT>
__device__ __forceinline__ Pack st_load(const SpanState<IdxT> &sp, int64_t l)
{
    Pack p;
    p.lo = st_ld<IdxT>(sp.xq + l * sp.KQ);
    p.hi = sp.KQ > 1 ? st_ld<IdxT>(sp.xq + l * sp.KQ + 1) : 0ull;
    return p;
}

// Layout of one span's node state at `base` (L nodes, KQ count words each):
// counts, then parent ids; the times and seek counters are bound per span.
template <typename IdxT>
__device__ __forceinline__ SpanState<IdxT> span_state_at(unsigned char *base, int64_t L, int KQ)
{
    SpanState<IdxT> sp;
    sp.KQ = KQ;
    sp.time = nullptr;
    sp.cnt = nullptr;
    sp.xq = (uint64_t *) base;
    sp.par = (IdxT *) (sp.xq + L * KQ);
    return sp;
}

// end of the state area (8-byte aligned), for kernels that add arrays
template <typename IdxT>
__device__ __forceinline__ unsigned char *span_state_end(const SpanState<IdxT> &sp, int64_t L)
{
    return (unsigned char *) (((uintptr_t) (sp.par + L) + 7) & ~(uintptr_t) 7);
}

// Rebuild the tree at a span's start in the span state (all threads of the
// block): every stateful node starts as a root carrying its own sample-set
// bits; the alive edges set the parents; counts accumulate bottom-up.  Ends
// with the block synchronised.
template <int W, int KQ, typename IdxT>
__device__ void span_seek(const TSView &ts, const QueryDev &qd, int32_t *err,
    const SpanState<IdxT> &sp, int K, int32_t Ls, const int32_t *l2g, int64_t a0, int64_t a1)
{
    constexpr uint32_t TSG_NO_PARENT = SpanState<IdxT>::NONE;
    // ---- seek: local nodes start as roots carrying their own weights
    for (int32_t l = threadIdx.x; l < Ls; l += blockDim.x) {
        const int32_t g = l2g[l];
        sp.par[l] = (IdxT) TSG_NO_PARENT;
        sp.cnt[l] = 0;
        pk_store(sp, (int64_t) l, pk_from_mask<W>(qd.node_mask[g], K));
    }
    __syncthreads();
    for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        const int2 pc = ts.span_alive_enc[i];
        if (pc.y >= 0) {
            sp.par[pc.y] = (IdxT) pc.x;
        }
    }
    __syncthreads();
    // bottom-up counts: every node is added to its parent once, by the
    // last of the parent's children to complete (counter word per node:
    // children in the low half, arrivals in the high half)
    for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        const int2 pc = ts.span_alive_enc[i];
        atomicAdd(&sp.cnt[pc.x], 1u);
    }
    __syncthreads();
    for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        const int2 pc = ts.span_alive_enc[i];
        if (pc.y >= 0 && (st_ld32<IdxT>(&sp.cnt[pc.y]) & 0xFFFFu) != 0) {
            continue;  // an internal child: completed by its own children
        }
        Pack contrib = pc.y >= 0 ? st_load(sp, pc.y)
                                 : pk_from_mask<W>(qd.node_mask[-pc.y - 1], K);
        uint32_t v = (uint32_t) pc.x;
        for (int32_t guard = 0; v != TSG_NO_PARENT; guard++) {
            if (guard > Ls) {
                dev_error(err, DEV_PATH_TOO_LONG);
                break;
            }
            if (contrib.lo) {
                atomicAdd((unsigned long long *) &sp.xq[(int64_t) v * KQ], (unsigned long long) contrib.lo);
            }
            if (KQ > 1 && contrib.hi) {
                atomicAdd((unsigned long long *) &sp.xq[(int64_t) v * KQ + (KQ > 1 ? 1 : 0)],
                    (unsigned long long) contrib.hi);
            }
            __threadfence_block();
            const uint32_t old = atomicAdd(&sp.cnt[v], 0x10000u);
            if ((old >> 16) + 1 != (old & 0xFFFFu)) {
                break;
            }
            __threadfence_block();
            contrib.lo = *(volatile unsigned long long *) &sp.xq[(int64_t) v * KQ];
            if (KQ > 1) {
                contrib.hi = *(volatile unsigned long long *) &sp.xq[(int64_t) v * KQ + (KQ > 1 ? 1 : 0)];
            }
            v = sp.par[v];
        }
    }
    __syncthreads();
}

}  // namespace tsg
