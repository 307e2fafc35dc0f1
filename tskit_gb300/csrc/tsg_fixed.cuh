// Exact accumulation of non-negative FP64 terms in 256-bit fixed point
// (2^-128 resolution), order-independent under atomic adds.
#pragma once

#include "tsg_internal.cuh"

namespace tsg {

#define TSG_FX_LIMBS 8
#define TSG_FX_FRAC 128

// Add v >= 0 to a fixed-point counter: v's 53-bit significand, placed at its
// binary position (2^-128 units; bits below are dropped), lands in at most
// three 32-bit limbs, each added to its own 64-bit counter (no carries, so
// the adds commute; at most 2^31 adds per counter).
__device__ __forceinline__ void fx_add(unsigned long long *acc, double v, int32_t *err)
{
    if (!(v > 0)) {
        return;
    }
    const unsigned long long bits = (unsigned long long) __double_as_longlong(v);
    int e = (int) (bits >> 52);
    unsigned long long m = bits & ((1ull << 52) - 1ull);
    if (e == 0x7FF) {
        dev_error(err, DEV_AFS_RANGE);
        return;
    }
    if (e != 0) {
        m |= 1ull << 52;
    } else {
        e = 1;
    }
    int shift = e - 1075 + TSG_FX_FRAC;
    if (shift < 0) {
        if (shift <= -53) {
            return;
        }
        m >>= -shift;
        shift = 0;
    }
    const int b = shift >> 5, r = shift & 31;
    if (b + 2 >= TSG_FX_LIMBS) {
        dev_error(err, DEV_AFS_RANGE);
        return;
    }
    const unsigned long long lo = (m & 0xFFFFFFFFull) << r;
    const unsigned long long hi = (m >> 32) << r;
    const unsigned long long l0 = lo & 0xFFFFFFFFull;
    const unsigned long long l1 = (lo >> 32) + (hi & 0xFFFFFFFFull);
    const unsigned long long l2 = hi >> 32;
    if (l0) {
        atomicAdd(acc + b, l0);
    }
    if (l1) {
        atomicAdd(acc + b + 1, l1);
    }
    if (l2) {
        atomicAdd(acc + b + 2, l2);
    }
}

// A non-negative integer held in n 32-bit limbs (least significant first),
// times 2^-TSG_FX_FRAC, rounded once to FP64 (round to nearest even: the
// top 64 bits below the leading one are kept and every lower bit folds into a
// sticky bit, which the single integer-to-double conversion then rounds
// correctly).
__device__ __forceinline__ double fx_round_limbs(const uint32_t *limb, int n)
{
    int top = n - 1;
    while (top >= 0 && limb[top] == 0) {
        top--;
    }
    if (top < 0) {
        return 0.0;
    }
    const unsigned long long hi =
        ((unsigned long long) limb[top] << 32) | (top >= 1 ? limb[top - 1] : 0u);
    const uint32_t nx = top >= 2 ? limb[top - 2] : 0u;
    bool sticky = false;
    for (int i = 0; i < top - 2; i++) {
        sticky |= limb[i] != 0;
    }
    const int sh = __clzll((long long) hi);
    unsigned long long m = hi;
    if (sh > 0) {
        m = (hi << sh) | ((unsigned long long) nx >> (32 - sh));
        sticky |= (uint32_t) (nx << sh) != 0u;
    } else {
        sticky |= nx != 0u;
    }
    // a sticky bit below the rounding position keeps round-to-nearest exact
    m |= sticky ? 1ull : 0ull;
    return ldexp(__ull2double_rn(m), 32 * (top - 1) - sh - TSG_FX_FRAC);
}

// The counter's exact value rounded once to FP64.
__device__ __forceinline__ double fx_value(const unsigned long long *acc)
{
    uint32_t limb[TSG_FX_LIMBS + 2];
    unsigned long long carry = 0;
#pragma unroll
    for (int i = 0; i < TSG_FX_LIMBS; i++) {
        const unsigned long long s = acc[i] + carry;
        const unsigned long long ov = s < carry ? 1ull : 0ull;
        limb[i] = (uint32_t) s;
        carry = (s >> 32) + (ov << 32);
    }
    limb[TSG_FX_LIMBS] = (uint32_t) carry;
    limb[TSG_FX_LIMBS + 1] = (uint32_t) (carry >> 32);
    return fx_round_limbs(limb, TSG_FX_LIMBS + 2);
}

// The exact difference a - b of two counters, rounded once to FP64: the
// limb-wise differences are normalised into 32-bit limbs with a signed top
// limb, a negative result is negated (two's complement over all limbs) and
// the magnitude rounded as fx_value rounds.
__device__ __forceinline__ double fx_diff_value(const unsigned long long *a,
    const unsigned long long *b)
{
    long long run[TSG_FX_LIMBS + 2];
    for (int i = 0; i < TSG_FX_LIMBS; i++) {
        run[i] = (long long) a[i] - (long long) b[i];
    }
    run[TSG_FX_LIMBS] = run[TSG_FX_LIMBS + 1] = 0;
    for (int i = 0; i < TSG_FX_LIMBS + 1; i++) {
        const long long cy = run[i] >> 32;
        run[i] -= cy * (1ll << 32);
        run[i + 1] += cy;
    }
    const bool neg = run[TSG_FX_LIMBS + 1] < 0;
    uint32_t limb[TSG_FX_LIMBS + 2];
    unsigned long long c = 1;
    for (int i = 0; i < TSG_FX_LIMBS + 2; i++) {
        const uint32_t v = (uint32_t) run[i];
        if (neg) {
            const unsigned long long t = (unsigned long long) (uint32_t) ~v + c;
            limb[i] = (uint32_t) t;
            c = t >> 32;
        } else {
            limb[i] = v;
        }
    }
    const double mag = fx_round_limbs(limb, TSG_FX_LIMBS + 2);
    return neg ? -mag : mag;
}

}  // namespace tsg
