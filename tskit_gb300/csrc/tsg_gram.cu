// Exact Gram matrix of a 0/1 genotype operand on the 5th-generation tensor
// cores (tcgen05), the one dense contraction of the statistics path.
//
// P = G G^T for G (rows = samples, K contiguous) holding 0 or 1 as FP8 E4M3
// bytes.  Products of 0/1 are exact and FP32 accumulation of at most 2^24
// of them is exact, so every tile is an exact integer; the caller splits K
// into chunks of at most 2^24 and the epilogue adds chunks (and a per-launch
// integer multiplier) into an int32 result.  (tcgen05.mma .kind::i8 is not
// available for sm_103a; .kind::f8f6f4 computes the same integers.)
//
// One CTA per 256 x 256 output tile of the upper triangle (block row <=
// block column), two 128-row halves sharing the B operand -- half the
// L2-to-SM operand bytes per FLOP of separate 128 x 256 tiles, the bound of
// this contraction:
//   warp 0       TMA producer: two 128 x 128-byte A tiles and one 256 x
//                128-byte B tile, 128-byte swizzle, into a 3-stage
//                shared-memory ring (mbarrier full/empty pairs);
//   warp 1       allocates all 512 TMEM columns (two FP32 accumulators of
//                256 columns, row = lane) and issues tcgen05.mma (M 128,
//                N 256, K 32) twice per K step, one per half, from one thread;
//                tcgen05.commit frees each stage and finally signals the
//                accumulators;
//   warps 2..5   epilogue: tcgen05.ld 32 lanes x 32 columns at a time, both
//                halves, convert to integers, add into the result.
// Every wait is bounded: on expiry the CTA records an error, drains its own
// copies in flight, frees its TMEM and returns.
#include <cuda.h>

#include "tsg_internal.cuh"

namespace tsg {

#define GRAM_BM 128                // rows of one MMA (one half of a tile)
#define GRAM_HALVES 2              // halves of a tile sharing the B operand
#define GRAM_TILE_ROWS (GRAM_BM * GRAM_HALVES)
#define GRAM_BN 256
#define GRAM_BK 128
#define GRAM_STAGES 3
#define GRAM_A_BYTES (GRAM_BM * GRAM_BK)
#define GRAM_B_BYTES (GRAM_BN * GRAM_BK)
#define GRAM_STAGE_BYTES (GRAM_HALVES * GRAM_A_BYTES + GRAM_B_BYTES)
#define GRAM_SMEM_BYTES (GRAM_STAGES * GRAM_STAGE_BYTES + 1024 + 256)
#define GRAM_TMEM_COLS (GRAM_HALVES * GRAM_BN)
#define GRAM_SPIN_LIMIT (1u << 26)

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the phase of parity `parity`; false on expiry
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (uint32_t i = 0; i < GRAM_SPIN_LIMIT; i++) {
        if (mbar_try_wait(bar, parity)) {
            return true;
        }
        if (i > 64) {
            __nanosleep(64);
        }
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int32_t x,
    int32_t y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"((uint64_t) map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// tcgen05 shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row
// groups 1024 bytes apart
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t) ((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t) 1 << 16;              // leading byte offset (unused for this layout)
    d |= (uint64_t) (1024 >> 4) << 32;    // stride byte offset
    d |= (uint64_t) 1 << 46;              // descriptor version
    d |= (uint64_t) 2 << 61;              // 128-byte swizzle
    return d;
}

// instruction descriptor: FP32 accumulator, E4M3 x E4M3, both K-major,
// N = 256, M = 128
__device__ __forceinline__ uint32_t umma_idesc()
{
    return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t) (GRAM_BN >> 3) << 17)
        | ((uint32_t) (GRAM_BM >> 4) << 24);
}

__device__ __forceinline__ void umma_f8(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
    uint32_t accumulate)
{
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

struct GramTile {
    int32_t row, col;  // first row and column of the tile
};

__global__ void __launch_bounds__(192, 1) k_gram_f8(const __grid_constant__ CUtensorMap mapA,
    const __grid_constant__ CUtensorMap mapB, const GramTile *tiles, int32_t n, int32_t kblocks,
    int32_t multiplier, int32_t accumulate_out, int32_t *P, int64_t ldp, int32_t *err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
    uint64_t *bars = (uint64_t *) (smem + GRAM_STAGES * GRAM_STAGE_BYTES);
    // bars[0..S): full, bars[S..2S): empty, bars[2S]: accumulator ready
    uint32_t *tmem_slot = (uint32_t *) (bars + 2 * GRAM_STAGES + 1);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const GramTile tile = tiles[blockIdx.x];

    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < GRAM_STAGES; s++) {
            mbar_init(smem_addr(&bars[s]), 1);
            mbar_init(smem_addr(&bars[GRAM_STAGES + s]), 1);
        }
        mbar_init(smem_addr(&bars[2 * GRAM_STAGES]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(tmem_slot)),
            "r"(GRAM_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *(volatile uint32_t *) tmem_slot;

    int issued = 0;  // producer: stages armed
    if (warp == 0) {
        if (lane == 0) {
            for (int kb = 0; kb < kblocks; kb++) {
                const int s = kb % GRAM_STAGES;
                const uint32_t round = (uint32_t) (kb / GRAM_STAGES);
                if (!mbar_wait(smem_addr(&bars[GRAM_STAGES + s]), (round & 1u) ^ 1u)) {
                    atomicExch(&s_abort, 1);
                    dev_error(err, 1);
                    break;
                }
                if (*(volatile int *) &s_abort) {
                    break;
                }
                const uint32_t full = smem_addr(&bars[s]);
                const uint32_t sa = smem_addr(smem + s * GRAM_STAGE_BYTES);
                mbar_expect_tx(full, GRAM_STAGE_BYTES);
                // rows past n (a last half outside the matrix) arrive as zeros
                tma_load_2d(sa, &mapA, kb * GRAM_BK, tile.row, full);
                tma_load_2d(sa + GRAM_A_BYTES, &mapA, kb * GRAM_BK, tile.row + GRAM_BM, full);
                tma_load_2d(sa + GRAM_HALVES * GRAM_A_BYTES, &mapB, kb * GRAM_BK, tile.col, full);
                issued = kb + 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = umma_idesc();
            bool ok = true;
            for (int kb = 0; kb < kblocks; kb++) {
                const int s = kb % GRAM_STAGES;
                const uint32_t round = (uint32_t) (kb / GRAM_STAGES);
                if (!mbar_wait(smem_addr(&bars[s]), round & 1u) || *(volatile int *) &s_abort) {
                    atomicExch(&s_abort, 1);
                    dev_error(err, 1);
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa = smem_addr(smem + s * GRAM_STAGE_BYTES);
                const uint64_t da0 = umma_desc(sa), da1 = umma_desc(sa + GRAM_A_BYTES);
                const uint64_t db = umma_desc(sa + GRAM_HALVES * GRAM_A_BYTES);
#pragma unroll
                for (int k = 0; k < GRAM_BK / 32; k++) {
                    // 32 E4M3 = 32 bytes along K: advance the start address;
                    // the second half accumulates 256 TMEM columns further
                    const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
                    umma_f8(tmem, da0 + (uint64_t) (k * 2), db + (uint64_t) (k * 2), idesc, acc);
                    umma_f8(tmem + GRAM_BN, da1 + (uint64_t) (k * 2), db + (uint64_t) (k * 2), idesc,
                        acc);
                }
                umma_commit(smem_addr(&bars[GRAM_STAGES + s]));
            }
            // the accumulator barrier fires once every issued MMA is done (or
            // at once if none was)
            umma_commit(smem_addr(&bars[2 * GRAM_STAGES]));
            (void) ok;
        }
    } else {
        // epilogue: warps 2..5 own TMEM lanes 32 * (warp % 4) ...
        const int quarter = warp & 3;
        const bool ready = mbar_wait(smem_addr(&bars[2 * GRAM_STAGES]), 0);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!ready) {
            atomicExch(&s_abort, 1);
            dev_error(err, 1);
        } else if (!*(volatile int *) &s_abort) {
#pragma unroll 1
          for (int h = 0; h < GRAM_HALVES; h++) {
            const int row = tile.row + h * GRAM_BM + quarter * 32 + lane;
#pragma unroll 1
            for (int c0 = 0; c0 < GRAM_BN; c0 += 32) {
                uint32_t v[32];
                const uint32_t taddr = tmem + ((uint32_t) (quarter * 32) << 16)
                    + (uint32_t) (h * GRAM_BN + c0);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                    "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                    "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, "
                    "%31}, [%32];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                    "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                    "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
                    "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                    "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]),
                    "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (row < n) {
                    int32_t *out = P + (int64_t) row * ldp + tile.col + c0;
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const int col = tile.col + c0 + j;
                        if (col < n) {
                            const int32_t x = (int32_t) __float2int_rn(__uint_as_float(v[j]))
                                * multiplier;
                            out[j] = accumulate_out ? out[j] + x : x;
                        }
                    }
                }
            }
          }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0 && lane == 0 && s_abort) {
        // drain copies armed but not consumed before the shared memory goes
        for (int kb = issued - GRAM_STAGES < 0 ? 0 : issued - GRAM_STAGES; kb < issued; kb++) {
            mbar_wait(smem_addr(&bars[kb % GRAM_STAGES]), (uint32_t) (kb / GRAM_STAGES) & 1u);
        }
    }
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
            "r"(GRAM_TMEM_COLS)
                     : "memory");
    }
}

// ------------------------------------------------------------------ host
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
    const cuuint64_t *, const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
    CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
    CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q)
                == cudaSuccess
            && q == cudaDriverEntryPointSuccess) {
            fn = (EncodeTiledFn) p;
        }
        cudaGetLastError();
    });
    return fn;
}

static int make_map(CUtensorMap *map, const uint8_t *G, int64_t rows, int64_t ld, int64_t kcols,
    uint32_t box_rows)
{
    EncodeTiledFn fn = encode_fn();
    if (fn == nullptr) {
        return TSG_ERR_CUDA;
    }
    cuuint64_t dims[2] = { (cuuint64_t) kcols, (cuuint64_t) rows };
    cuuint64_t strides[1] = { (cuuint64_t) ld };
    cuuint32_t box[2] = { GRAM_BK, box_rows };
    cuuint32_t estr[2] = { 1, 1 };
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void *) G, dims, strides, box, estr,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : TSG_ERR_CUDA;
}

// Tiles of the upper triangle: 256 x 256 blocks (row block <= column
// block), row-major order; together they hold every entry (i, j), i <= j.
int gram_tiles(int64_t n, std::vector<int32_t> &out)
{
    out.clear();
    for (int64_t r = 0; r < n; r += GRAM_TILE_ROWS) {
        for (int64_t c = r; c < n; c += GRAM_BN) {
            out.push_back((int32_t) r);
            out.push_back((int32_t) c);
        }
    }
    return 0;
}

// P (+)= multiplier * G G^T over the upper-triangle tiles, where G is
// rows x ld bytes (E4M3 0/1, K contiguous; kcols <= 2^24 used, a multiple of
// 128; ld a multiple of 16, G 16-byte aligned).  tiles: device copy of
// gram_tiles(n).
int launch_gram(const uint8_t *G, int64_t n, int64_t ld, int64_t k0, int64_t kcols,
    const int32_t *tiles, int64_t num_tiles, int32_t multiplier, bool accumulate, int32_t *P,
    int64_t ldp, int32_t *err, cudaStream_t st)
{
    if (kcols <= 0 || num_tiles == 0) {
        return 0;
    }
    if (kcols > ((int64_t) 1 << 24) || kcols % GRAM_BK != 0 || k0 % GRAM_BK != 0 || ld % 16 != 0
        || ((uintptr_t) G & 15u) != 0) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    CUtensorMap mapA, mapB;
    int ret;
    const uint8_t *base = G + k0;
    if ((ret = make_map(&mapA, base, n, ld, kcols, GRAM_BM)) != 0
        || (ret = make_map(&mapB, base, n, ld, kcols, GRAM_BN)) != 0) {
        return ret;
    }
    static std::once_flag once;
    std::call_once(once, []() {
        cudaFuncSetAttribute(k_gram_f8, cudaFuncAttributeMaxDynamicSharedMemorySize,
            GRAM_SMEM_BYTES);
    });
    k_gram_f8<<<(unsigned) num_tiles, 192, GRAM_SMEM_BYTES, st>>>(mapA, mapB,
        (const GramTile *) tiles, (int32_t) n, (int32_t) (kcols / GRAM_BK), multiplier,
        accumulate ? 1 : 0, P, ldp, err);
    TSG_LAUNCHED();
    return 0;
}

}  // namespace tsg
