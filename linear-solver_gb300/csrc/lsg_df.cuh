// lsg_df.cuh — double-float (two FP32 words) evaluation of the FP64 stencil.
//
// GB300 runs FP64 arithmetic at ~1/64 of its FP32 rate (2 FP64 lanes per
// clock per SM), and the 37-point periodic stencil of MPI_REAL/system.c:189-204
// needs ~44 FP64 operations per point, so an FP64 stencil pass is bound by
// the FP64 pipe at ~9x its HBM time.  The FP64 stencil passes of the solvers
// therefore evaluate Au in double-float arithmetic on the FP32 pipe:
//
//   * each double entering the march is split once, with integer and FP32
//     operations only, into hi = the value truncated to 24 significant bits
//     and lo = the remaining 29 bits rounded to 24 (relative error 2^-49;
//     hi + lo is itself a double, exactly);
//   * the six neighbours at distance p are summed with Knuth's error-free
//     TwoSum on the hi words (the rounding error of every FP32 addition is
//     recovered exactly) and plain FP32 sums of the lo words and errors;
//   * the weights w_p are three floats summing to the double exactly; S_p w_p
//     is formed with the FMA two-product (Dekker's product with a fused
//     multiply-add) and accumulated by TwoSum;
//   * results are rounded back to doubles with integer operations.
//
// The result agrees with an FP64 evaluation to ~2^-48 of sum_p |w_p| |u|
// (FP64's own rounding is ~2^-53 of it).  Values are scaled by a power of
// two 2^k before the split (k from the solve's ||b||), so the float exponent
// range covers |u| from 2^-74 to 2^127 times 2^-k at full precision; a finite
// value above that range raises the solve's df_range flag (status
// LSG_RANGE), values below it lose their lo word.
//
// References: T. J. Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18 (1971); D. E. Knuth, TAOCP vol. 2,
// 4.2.2 (TwoSum).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace lsg {

// Exponent shift k applied before the split: ||b|| 2^k in [1, 2), clamped
// to |k| <= 700 so every rebias below stays inside the double exponent range
// (a right-hand side beyond 2^+-700 pushes values out of the float range,
// which raises the flag).
__host__ __device__ inline int df_shift_for(double rhs_norm) {
    if (!(rhs_norm > 0.0) || !(rhs_norm < INFINITY)) return 0;
    int e = 0;
    frexp(rhs_norm, &e);  // rhs_norm = f 2^e, f in [0.5, 1)
    const int k = 1 - e;
    return k > 700 ? 700 : (k < -700 ? -700 : k);
}

// s + e = a + b exactly (Knuth's TwoSum; no ordering assumption).
__device__ __forceinline__ void df_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Splits u 2^k into (hi, lo) floats.  hi: the sign, exponent and the top 24
// significant bits of u (truncated); lo: the low 29 bits of the significand,
// rounded to a float of the same sign.  NaN / Inf give a NaN hi word (so the
// solve's NaN detection still fires); a finite value too large for the float
// range sets `bad`; one too small flushes to zero.
__device__ __forceinline__ float2 df_split(double u, int k, bool &bad) {
    const unsigned H = (unsigned)__double2hiint(u), L = (unsigned)__double2loint(u);
    const int e11 = (int)((H >> 20) & 0x7ffu);
    const int es = e11 + k;                  // biased exponent of u 2^k
    const unsigned sign = H & 0x80000000u;
    const unsigned m23 = __funnelshift_l(L, H, 3) & 0x7fffffu;  // significand bits 51..29
    float hi = __uint_as_float(sign | ((unsigned)(es - 896) << 23) | m23);
    // lo = u 2^k - hi = rem 2^(es - 1075), rem = L & (2^29 - 1), same sign as
    // u.  rem = a 2^23 + b (a < 64, b < 2^23) is converted without an
    // integer-to-float instruction (which runs on the slow conversion unit):
    // a float with exponent E and significand field b is 2^E + b 2^(E - 23),
    // so subtracting 2^E leaves b 2^(E - 23) exactly; likewise for a, placed
    // in the top six significand bits.  The final addition rounds once.
    const unsigned eb = (unsigned)(es - 925) << 23;   // b 2^(es - 1075): E = es - 1052
    const unsigned ea = eb + (6u << 23);               // a 2^(es - 1052): E = es - 1046
    const float xb = __fsub_rn(__uint_as_float(eb | (L & 0x7fffffu)), __uint_as_float(eb));
    const float xa = __fsub_rn(__uint_as_float(ea | ((L >> 6) & 0x7e0000u)), __uint_as_float(ea));
    float lo = __uint_as_float(__float_as_uint(__fadd_rn(xa, xb)) | sign);
    if (es < 949) lo = __uint_as_float(sign);  // below 2^-74: the lo word underflows
    if (es < 897 || es > 1150) {             // outside the normal float range
        if (e11 == 2047) {
            hi = __uint_as_float(0x7fc00000u);
        } else {
            bad |= es > 1150;
            hi = __uint_as_float(sign);
        }
        lo = __uint_as_float(sign);
    }
    return make_float2(hi, lo);
}

// The double equal to f 2^-k (f a float; denormal floats read as zero;
// |k| <= 700 keeps the rebiased exponent in range).  Integer operations
// only: exponent rebias and significand shift.
__device__ __forceinline__ double df_f2d(float f, int k) {
    const unsigned b = __float_as_uint(f);
    const unsigned a = b & 0x7fffffffu;
    unsigned hi = (a >> 3) + ((unsigned)(896 - k) << 20);
    unsigned lo = b << 29;
    if (a < 0x00800000u) hi = 0u, lo = 0u;          // zero / denormal
    if (a >= 0x7f800000u) hi = 0x7ff80000u, lo = 0u;  // NaN / Inf stay non-finite
    return __hiloint2double((int)(hi | (b & 0x80000000u)), (int)lo);
}

// (hi + lo) 2^-k as a double: the pair is renormalised (|lo| <= ulp(hi) / 2),
// then converted with integer operations only: hi's bit pattern as a double plus lo counted
// in units of that double's last place (the pattern is monotonic, so the
// addition carries into the exponent correctly).  lo's bits below that place
// are truncated (an error below one unit in the last place of the double).
// When hi is an exact power of two and lo has the opposite sign the result
// lies in the binade below, whose unit is half as large.
__device__ __forceinline__ double df_to_double(float2 v, int k) {
    {  // renormalise (Fast2Sum: |hi| >= |lo| for every pair formed here)
        const float h = __fadd_rn(v.x, v.y);
        v.y = __fsub_rn(v.y, __fsub_rn(h, v.x));
        v.x = h;
    }
    // every case as an integer bit pattern, one reinterpretation at the end
    const unsigned bh = __float_as_uint(v.x), bl = __float_as_uint(v.y);
    const unsigned ah = bh & 0x7fffffffu, al = bl & 0x7fffffffu;
    const unsigned H = (ah >> 3) + ((unsigned)(896 - k) << 20);
    const int sh = (int)(al >> 23) - (int)(ah >> 23) + 29;  // lo's unit exponent minus the double's
    const unsigned ml = (al & 0x7fffffu) | 0x800000u;
    unsigned t = sh >= 0 ? (ml << (sh > 7 ? 7 : sh)) : (sh > -25 ? (ml >> -sh) : 0u);
    t = al < 0x00800000u ? 0u : t;
    const unsigned opp = (bh ^ bl) >> 31;
    t = (opp && (ah & 0x7fffffu) == 0u) ? t << 1 : t;
    const unsigned long long P = ((unsigned long long)H << 32) | (bh << 29);
    unsigned long long R = (opp ? P - t : P + t) | ((unsigned long long)(bh & 0x80000000u) << 32);
    // hi zero (or denormal): lo alone, as df_f2d forms it
    const unsigned HL = al < 0x00800000u ? 0u : (al >> 3) + ((unsigned)(896 - k) << 20);
    const unsigned LL = al < 0x00800000u ? 0u : bl << 29;
    const unsigned long long RL = ((unsigned long long)(HL | (bl & 0x80000000u)) << 32) | LL;
    R = ah < 0x00800000u ? RL : R;
    R = ah >= 0x7f800000u ? 0x7ff8000000000000ull : R;
    return __longlong_as_double((long long)R);
}

// Double-float pair of a double constant: hi = the float nearest w, lo = the
// float nearest w - hi.
__host__ __device__ inline float2 df_weight(double w) {
    const float h = (float)w;
    const float l = (float)(w - (double)h);
    return make_float2(h, l);
}

// Double-float accumulator: acc += S w, S = (sh, sl), w = w1 + w2 + w3 (the
// double weight exactly; w3 contributes ~2^-48 of the product).
__device__ __forceinline__ void df_fma_acc(float2 &acc, float sh, float sl, float w1, float w2, float w3) {
    const float ph = __fmul_rn(sh, w1);
    float pe = __fmaf_rn(sh, w1, -ph);  // exact error of sh * w1
    pe = __fmaf_rn(sh, w2, pe);
    pe = __fmaf_rn(sl, w1, pe);
    pe = __fmaf_rn(sh, w3, pe);
    float s, e;
    df_two_sum(acc.x, ph, s, e);
    acc.x = s;
    acc.y = __fadd_rn(acc.y, __fadd_rn(pe, e));
}

// a + b, the hi addition error-free, the lo word left unnormalised (it stays
// ~2^-24 of the hi word through the few additions of one stencil sum).
__device__ __forceinline__ float2 df_add2(float2 a, float2 b) {
    float s, e;
    df_two_sum(a.x, b.x, s, e);
    return make_float2(s, __fadd_rn(__fadd_rn(a.y, b.y), e));
}

// a - b, renormalised (hi = the float nearest the pair's sum) by a second
// TwoSum: near convergence b - Au cancels to a few bits of the hi words.
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) {
    float s, e;
    df_two_sum(a.x, -b.x, s, e);
    e = __fadd_rn(e, __fsub_rn(a.y, b.y));
    float h, l;
    df_two_sum(s, e, h, l);
    return make_float2(h, l);
}

// a + b, renormalised.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) { return df_sub(a, make_float2(-b.x, -b.y)); }

// a c for a double-float constant c = (ch, cl), renormalised.
__device__ __forceinline__ float2 df_mul(float2 a, float2 c) {
    const float p = __fmul_rn(a.x, c.x);
    float e = __fmaf_rn(a.x, c.x, -p);
    e = __fmaf_rn(a.x, c.y, e);
    e = __fmaf_rn(a.y, c.x, e);
    const float h = __fadd_rn(p, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, p)));  // |e| << |p|: fast renormalisation
}

}  // namespace lsg
