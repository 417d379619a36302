// Exact IEEE-754 binary64 squaring and accumulation on the integer pipes.
//
// GB300's FP64 pipe is a small fraction of its FP32/INT32 throughput, and the
// float64 distance kernel (three FP64 operations per coordinate: subtract,
// square, add) runs at that pipe's limit.  sqr_rn(d) returns the correctly
// rounded (round-to-nearest-even) square of d computed with 32x32->64-bit
// integer products, so the square moves to the integer pipes; sqr_add_rn(acc,
// d) returns RN(acc + RN(d*d)) the same way, the square never packed into a
// double, and the distance kernel applies it to 12 of its 16 accumulators so
// that the FP64 pipe (the subtraction and the other 4 sums) and the integer
// pipes carry balanced loads.  The square's result is bit-identical to d*d
// under IEEE-754 for every input: zero returns +0, and values whose square is
// not a normal double (|d| < 2^-511 or |d| >= 2^511, subnormals, infinities,
// NaN) take the hardware multiply behind a warp-uniform branch, so no FP64
// multiply is issued while every lane of the warp is on the integer path.
//
// Method (the textbook integer multiply of two binary64 significands):
//   d = m * 2^(e-1075), m = 2^52 | fraction (53 bits), e the biased exponent;
//   m^2 = mh^2 * 2^64 + 2*mh*ml * 2^32 + ml^2 with mh the top 21 and ml the
//   low 32 bits of m, so m^2 in [2^104, 2^106) is exact in 128 bits; adding
//   2^(51+top) - 1 + (lowest kept bit) and truncating to the top 53 bits
//   rounds it to nearest-even (top = 1 when m^2 >= 2^105), and the biased
//   exponent of d^2 is 2e - 1023 + top; a rounding carry into bit 53 moves
//   into the exponent field by the addition that packs the result.  On the
//   device the three products are mul.wide.u32, the 128-bit sums add.cc/addc
//   chains, and extracting the significand one funnel shift per word.
// Usable from host code (tests compare it with the host's multiply and add).
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define HDB_HD __host__ __device__ __forceinline__
#else
#define HDB_HD inline
#endif

namespace hdb {

HDB_HD uint64_t exact_bits(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    std::memcpy(&b, &d, sizeof(b));
    return b;
#endif
}

HDB_HD double exact_double(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
#endif
}

// 32-bit word primitives.  On GB300 64-bit integer adds, shifts and compares
// are issued to the FP64 pipe, which is exactly the pipe being relieved, so
// the square is written with 32-bit operations only.
HDB_HD void mul_wide(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#ifdef __CUDA_ARCH__
    asm("{\n\t.reg .b64 t;\n\tmul.wide.u32 t, %2, %3;\n\tmov.b64 {%0, %1}, t;\n\t}" : "=r"(lo), "=r"(hi) : "r"(a), "r"(b));
#else
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    lo = (uint32_t)p;
    hi = (uint32_t)(p >> 32);
#endif
}

// r = a + b + carry_in, carry_out in {0, 1}.
HDB_HD uint32_t add_carry(uint32_t a, uint32_t b, uint32_t carry_in, uint32_t& carry_out) {
    const uint32_t t = a + b;
    const uint32_t c1 = t < a ? 1u : 0u;
    const uint32_t r = t + carry_in;
    carry_out = c1 | (r < t ? 1u : 0u);
    return r;
}

// (hi:lo) += (bh:bl), two-word add with the carry between the words.
HDB_HD void add2(uint32_t& lo, uint32_t& hi, uint32_t bl, uint32_t bh) {
#ifdef __CUDA_ARCH__
    asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(lo), "+r"(hi) : "r"(bl), "r"(bh));
#else
    uint32_t c;
    lo = add_carry(lo, bl, 0u, c);
    hi = hi + bh + c;
#endif
}

// (w3:w2:w1) = (c:b2:b1) + (0:a2:a1), three-word add with carries.
HDB_HD void add3(uint32_t a1, uint32_t b1, uint32_t a2, uint32_t b2, uint32_t c, uint32_t& w1, uint32_t& w2,
                 uint32_t& w3) {
#ifdef __CUDA_ARCH__
    asm("add.cc.u32 %0, %3, %4;\n\taddc.cc.u32 %1, %5, %6;\n\taddc.u32 %2, %7, 0;"
        : "=r"(w1), "=r"(w2), "=r"(w3)
        : "r"(a1), "r"(b1), "r"(a2), "r"(b2), "r"(c));
#else
    uint32_t c1, c2;
    w1 = add_carry(a1, b1, 0u, c1);
    w2 = add_carry(a2, b2, c1, c2);
    w3 = c + c2;
#endif
}

// (hi:lo) >> s for 0 <= s < 32, low word.
HDB_HD uint32_t funnel_right(uint32_t lo, uint32_t hi, uint32_t s) {
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, s);
#else
    return s ? (lo >> s) | (hi << (32 - s)) : lo;
#endif
}

// (hi:lo) << s for 0 <= s < 32, high word.
HDB_HD uint32_t funnel_left(uint32_t lo, uint32_t hi, uint32_t s) {
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, s);
#else
    return s ? (hi << s) | (lo >> (32 - s)) : hi;
#endif
}

// x << n for 0 <= n <= 32 (0 when n == 32).
HDB_HD uint32_t shl_upto32(uint32_t x, uint32_t n) {
#ifdef __CUDA_ARCH__
    return __funnelshift_lc(0u, x, n);
#else
    return n < 32u ? x << n : 0u;
#endif
}

// (w3:w2:w1) += (0:0:k) + carry, the carry being that of w0 + 0xffffffff
// (1 exactly when w0 != 0).
HDB_HD void add_round(uint32_t w0, uint32_t k, uint32_t& w1, uint32_t& w2, uint32_t& w3) {
#ifdef __CUDA_ARCH__
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %3, 0xffffffff;\n\taddc.cc.u32 %0, %0, %4;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\taddc.u32 %2, %2, 0;\n\t}"
        : "+r"(w1), "+r"(w2), "+r"(w3)
        : "r"(w0), "r"(k));
#else
    uint32_t c = w0 != 0u ? 1u : 0u;
    w1 = add_carry(w1, k, c, c);
    w2 = add_carry(w2, 0u, c, c);
    w3 += c;
#endif
}

// Rounded significand of d^2 for d with biased exponent 512..1533 (garbage
// elsewhere): d^2 = (qh:ql) * 2^(eq - 1075) with (qh:ql) in [2^52, 2^53] (2^53
// when the rounding carries out) and eq the biased exponent of the exact
// square.  (hi, lo) are the two words of d.
HDB_HD void sqr_sig_words(uint32_t hi, uint32_t lo, uint32_t& qh, uint32_t& ql, uint32_t& eq) {
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const uint32_t mh = (hi & 0xfffffu) | 0x100000u;  // top 21 bits of m
    const uint32_t ml = lo;                           // low 32 bits of m
    uint32_t p0h, p0l, p1h, p1l, p2h, p2l;
    mul_wide(ml, ml, p0h, p0l);  // ml^2
    mul_wide(mh, ml, p1h, p1l);  // mh*ml < 2^53
    mul_wide(mh, mh, p2h, p2l);  // mh^2 < 2^42
    // S = m^2 = p2 * 2^64 + p1 * 2^33 + p0 in words w3:w2:w1:w0.
    uint32_t w1, w2, w3;
    add3(p0h, p1l << 1, p2l, funnel_left(p1l, p1h, 1u), p2h, w1, w2, w3);
    const uint32_t w0 = p0l;
    // S in [2^104, 2^106), so w3 < 2^10 and top = bit 105 = w3 >> 9.  The
    // significand is S >> (52 + top): bit sh of w1 is its lowest bit.  Round
    // to nearest-even by adding 2^(51 + top) - 1 + lsb before truncating:
    // (2^(19 + top) - 1) to w1 plus the carry of (w0 | lsb) + 0xffffffff.
    const uint32_t top = w3 >> 9;
    const uint32_t sh = 20u + top;
    const uint32_t lsb = (w1 >> sh) & 1u;
    add_round(w0 | lsb, top ? 0xfffffu : 0x7ffffu, w1, w2, w3);
    ql = funnel_right(w1, w2, sh);
    qh = funnel_right(w2, w3, sh);  // w3 < 2^11: no bits above the significand
    eq = 2u * e - 1023u + top;
}

// Integer part of sqr_rn; valid for biased exponents 512..1533 (every normal
// result) and for zero (returns +0), garbage elsewhere.  (hi, lo) are the two
// words of d; every select stays on 32-bit words (a double-typed select is an
// FP64-pipe instruction).
HDB_HD double sqr_rn_words(uint32_t hi, uint32_t lo, bool zero) {
    uint32_t qh, ql, eq;
    sqr_sig_words(hi, lo, qh, ql, eq);
    // (eq - 1) << 20 plus the high word (hidden bit included) packs the
    // result, a significand of 2^53 moving into the exponent field.
    const uint32_t rhi = zero ? 0u : ((eq - 1u) << 20) + qh;
    const uint32_t rlo = zero ? 0u : ql;
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)rhi, (int)rlo);
#else
    return exact_double(((uint64_t)rhi << 32) | rlo);
#endif
}

// RN(acc + RN(d * d)), both roundings to nearest-even, on the integer pipes,
// for the float64 distance accumulator: acc is +0 or a normal double below
// 2^1008 and d is 0 or has |d| in [2^-511, 2^501] (so d^2 is normal and the
// sum cannot overflow).  (ahi, alo) and (dhi, dlo) are the words of acc and d.
// The square stays unpacked (significand and exponent from sqr_sig_words);
// the operand with the larger exponent is x, the other y is shifted right by
// the exponent difference (clamped to 63: y < 2^54, so beyond that only its
// sticky bit matters) keeping the 32 bits below x's lowest bit (r, round bit
// at 31) and an OR of anything further (beyond); x + y has at most one carry
// bit, removed by a one-place shift; then round to nearest-even and pack.
HDB_HD void sqr_add_rn_words(uint32_t ahi, uint32_t alo, uint32_t dhi, uint32_t dlo, uint32_t& rhi,
                             uint32_t& rlo) {
    const bool dzero = ((dhi << 1) | dlo) == 0u;
    uint32_t qh, ql, eq;
    sqr_sig_words(dhi, dlo, qh, ql, eq);
    const uint32_t ea = ahi >> 20;  // 0 for +0
    const uint32_t mah = (ahi & 0xfffffu) | (ahi < 0x100000u ? ahi : 0x100000u);  // hidden bit unless +0
    const bool q_big = eq > ea;
    const uint32_t ex = q_big ? eq : ea;
    const uint32_t dist = q_big ? eq - ea : ea - eq;
    const uint32_t xh = q_big ? qh : mah, xl = q_big ? ql : alo;
    const uint32_t yh = q_big ? mah : qh, yl = q_big ? alo : ql;
    const uint32_t s = dist < 63u ? dist : 63u, sb = s & 31u;
    const bool big = s >= 32u;
    const uint32_t v = yh >> sb, u = funnel_right(yl, yh, sb), t = shl_upto32(yl, 32u - sb);
    const uint32_t bl = big ? v : u, bh = big ? 0u : v;  // y >> s
    const uint32_t r = big ? u : t, beyond = big ? t : 0u;
    uint32_t sl = xl, sh = xh;
    add2(sl, sh, bl, bh);
    const uint32_t c = sh >> 21;  // x + y >= 2^53
    uint32_t ml = funnel_right(sl, sh, c), mh = sh >> c;
    const uint32_t f = funnel_right(r, sl, c);  // the 32 bits below the result's lowest bit
    const uint32_t sticky = (f << 1) | (r & c) | beyond;
    const uint32_t up = (f >> 31) & ((sticky != 0u ? 1u : 0u) | ml);
    add2(ml, mh, up, 0u);
    rhi = dzero ? ahi : ((ex + c - 1u) << 20) + mh;
    rlo = dzero ? alo : ml;
}

HDB_HD double sqr_add_rn(double acc, double d) {
#ifdef __CUDA_ARCH__
    const uint32_t ahi = (uint32_t)__double2hiint(acc), alo = (uint32_t)__double2loint(acc);
    const uint32_t dhi = (uint32_t)__double2hiint(d), dlo = (uint32_t)__double2loint(d);
#else
    const uint64_t ab = exact_bits(acc), db = exact_bits(d);
    const uint32_t ahi = (uint32_t)(ab >> 32), alo = (uint32_t)ab, dhi = (uint32_t)(db >> 32), dlo = (uint32_t)db;
#endif
    uint32_t rhi, rlo;
    sqr_add_rn_words(ahi, alo, dhi, dlo, rhi, rlo);
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)rhi, (int)rlo);
#else
    return exact_double(((uint64_t)rhi << 32) | rlo);
#endif
}

// Domain of sqr_add_rn: coordinates 0 or with |x| in [2^-459, 2^500) (every
// difference is then 0 or in [2^-511, 2^501]) and accumulators +0 or normal
// below 2^1000 (16 more squares below 2^1002 keep the sum below 2^1008).
HDB_HD bool sqr_add_operand_safe(double x) {
#ifdef __CUDA_ARCH__
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
#else
    const uint64_t bits = exact_bits(x);
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
#endif
    const uint32_t e = (hi >> 20) & 0x7ffu;
    return (((hi << 1) | lo) == 0u) || (e >= 1023u - 459u && e < 1023u + 500u);
}

HDB_HD bool sqr_add_acc_safe(double acc) {
#ifdef __CUDA_ARCH__
    const uint32_t hi = (uint32_t)__double2hiint(acc), lo = (uint32_t)__double2loint(acc);
#else
    const uint64_t bits = exact_bits(acc);
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
#endif
    return (hi | lo) == 0u || (hi - 0x100000u) < ((1023u + 1000u) << 20) - 0x100000u;
}

// True when every difference a - b of two such values squares to a normal
// double (or is zero): |a|, |b| in {0} U [2^-459, 2^509) give |RN(a - b)| = 0
// or in [2^-511, 2^510], i.e. biased exponents 512..1533.
HDB_HD bool sqr_operand_safe(double x) {
#ifdef __CUDA_ARCH__
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
#else
    const uint64_t bits = exact_bits(x);
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
#endif
    const uint32_t e = (hi >> 20) & 0x7ffu;
    return (((hi << 1) | lo) == 0u) || (e >= 1023u - 459u && e < 1023u + 509u);
}

// Square of a difference of sqr_operand_safe values (no hardware fallback).
HDB_HD double sqr_rn_safe(double d) {
#ifdef __CUDA_ARCH__
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
#else
    const uint64_t bits = exact_bits(d);
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
#endif
    return sqr_rn_words(hi, lo, ((hi << 1) | lo) == 0u);
}

HDB_HD double sqr_rn(double d) {
#ifdef __CUDA_ARCH__
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
#else
    const uint64_t bits = exact_bits(d);
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
#endif
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const bool zero = ((hi << 1) | lo) == 0u;
    const bool hw = (e < 512u || e > 1533u) && !zero;  // square not a normal double
    double r = sqr_rn_words(hi, lo, zero);
#ifdef __CUDA_ARCH__
    // Full-warp callers only: the branch is taken by the whole warp or not at all.
    if (__any_sync(0xffffffffu, hw)) {
        if (hw) r = __dmul_rn(d, d);
    }
#else
    if (hw) r = d * d;
#endif
    return r;
}

}  // namespace hdb
