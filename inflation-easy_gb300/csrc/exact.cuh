// exact.cuh -- exact lattice sums and exact division by a fixed divisor, on
// the integer pipes.
//
// GB300 runs FP64 arithmetic at a small fraction of its integer and FP32
// rates, and the plain FP64 form must keep every per-site result bit-equal
// to IEEE double evaluation.  Two pieces of that work need no FP64 pipe:
//
// * Lattice sums (the Friedmann update's sum f*lapl(f) and potential sum).
//   A floating-point sum of N^3 terms depends on the order of its additions,
//   and the reference's serial loop order cannot be followed by a parallel
//   reduction.  Here every term is added exactly into a 256-bit two's-
//   complement fixed-point word (least significant bit 2^-192), words of
//   threads, warps and CTAs are added as integers, and the total is rounded
//   to the nearest double (ties to even) once.  The result is the correctly
//   rounded exact sum: independent of the launch shape and of the order of
//   the terms, and reproducible by any exact summation on the CPU.  A term
//   must be finite with magnitude below 2^30 (up to 2^32 terms cannot then
//   overflow); bits of a term below 2^-192 are dropped toward zero.  Lattice
//   terms never carry such bits in practice: a Laplacian of fields of order
//   0.01..10 is a multiple of their ulp (2^-59 or coarser).
//
//   The sums of products (f lapl(f), f^2, fd^2) add the exact 106-bit
//   product of the two significands, so the multiplication needs no FP64
//   pipe either: the total is the correctly rounded exact sum of the exact
//   products.
//
// * Division by a divisor fixed for the whole run (B^2 in V' = (c2 v)/B^2).
//   The correctly rounded quotient RN(x / y) is formed from the integer
//   quotient of the significands: with precomputed R = floor(2^116 / M_y)
//   (division by an invariant integer by multiplication, Granlund and
//   Montgomery, PLDI 1994), floor(M_x 2^s / M_y) is found exactly after at
//   most one correction from the remainder, and the remainder decides the
//   IEEE round-to-nearest-even rounding.  Zero, subnormal, infinite and NaN
//   operands, and quotients outside the normal range, take the native
//   division, so the result equals x / y for every x.
#pragma once

#include <stdint.h>

namespace iegpu {

__host__ __device__ __forceinline__ unsigned long long dbits(double x) {
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long b;
    __builtin_memcpy(&b, &x, sizeof b);
    return b;
#endif
}

__host__ __device__ __forceinline__ double bitsd(unsigned long long b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    __builtin_memcpy(&x, &b, sizeof x);
    return x;
#endif
}

// ---------------------------------------------------------------------------
// exact sums
// ---------------------------------------------------------------------------

struct Acc4 {
    unsigned long long w[4];   // little-endian limbs; value = (int256) w * 2^-192
};

constexpr int kAccShift = 883;          // biased exponent 1075 - 192
constexpr int kAccMaxExp = 1053;        // biased exponent of 2^30

__host__ __device__ __forceinline__ void acc_zero(Acc4& A) {
    A.w[0] = A.w[1] = A.w[2] = A.w[3] = 0ull;
}

__host__ __device__ __forceinline__ void acc_add4(Acc4& A, unsigned long long b0, unsigned long long b1,
                                                  unsigned long long b2, unsigned long long b3) {
#ifdef __CUDA_ARCH__
    asm("add.cc.u64 %0, %0, %4;\n\t"
        "addc.cc.u64 %1, %1, %5;\n\t"
        "addc.cc.u64 %2, %2, %6;\n\t"
        "addc.u64 %3, %3, %7;"
        : "+l"(A.w[0]), "+l"(A.w[1]), "+l"(A.w[2]), "+l"(A.w[3])
        : "l"(b0), "l"(b1), "l"(b2), "l"(b3));
#else
    const unsigned long long b[4] = {b0, b1, b2, b3};
    unsigned long long carry = 0;
    for (int q = 0; q < 4; ++q) {
        const unsigned long long t = A.w[q] + b[q];
        const unsigned long long c1 = t < b[q];
        A.w[q] = t + carry;
        carry = c1 | (A.w[q] < t);
    }
#endif
}

__host__ __device__ __forceinline__ void acc_sub4(Acc4& A, unsigned long long b0, unsigned long long b1,
                                                  unsigned long long b2, unsigned long long b3) {
#ifdef __CUDA_ARCH__
    asm("sub.cc.u64 %0, %0, %4;\n\t"
        "subc.cc.u64 %1, %1, %5;\n\t"
        "subc.cc.u64 %2, %2, %6;\n\t"
        "subc.u64 %3, %3, %7;"
        : "+l"(A.w[0]), "+l"(A.w[1]), "+l"(A.w[2]), "+l"(A.w[3])
        : "l"(b0), "l"(b1), "l"(b2), "l"(b3));
#else
    const unsigned long long b[4] = {b0, b1, b2, b3};
    unsigned long long borrow = 0;
    for (int q = 0; q < 4; ++q) {
        const unsigned long long t = A.w[q] - b[q];
        const unsigned long long c1 = A.w[q] < b[q];
        A.w[q] = t - borrow;
        borrow = c1 | (t < borrow);
    }
#endif
}

__host__ __device__ __forceinline__ void acc_add(Acc4& A, const Acc4& B) { acc_add4(A, B.w[0], B.w[1], B.w[2], B.w[3]); }

// Adds the double t exactly.  flags |= 1 for a non-finite term, 2 for a
// finite term of magnitude >= 2^30 (neither is added).
__host__ __device__ __forceinline__ void acc_add_term(Acc4& A, double t, unsigned& flags) {
    const unsigned long long b = dbits(t);
    int e = (int)((b >> 52) & 0x7FF);
    unsigned long long m = b & 0x000FFFFFFFFFFFFFull;
    if (e >= kAccMaxExp) {
        flags |= (e == 0x7FF) ? 1u : 2u;
        return;
    }
    if (e == 0) {
        if (m == 0) return;
        e = 1;
    } else {
        m |= 1ull << 52;
    }
    int s = e - kAccShift;   // bit position of m's lowest bit
    if (s < 0) {
        m = (s <= -64) ? 0ull : (m >> (-s));
        s = 0;
    }
    const int q = s >> 6, r = s & 63;   // q <= 2 since s <= 169
    const unsigned long long lo = m << r;
    const unsigned long long hi = r ? (m >> (64 - r)) : 0ull;
    const unsigned long long l0 = q == 0 ? lo : 0ull;
    const unsigned long long l1 = q == 0 ? hi : (q == 1 ? lo : 0ull);
    const unsigned long long l2 = q == 1 ? hi : (q == 2 ? lo : 0ull);
    const unsigned long long l3 = q == 2 ? hi : 0ull;
    if (b >> 63) acc_sub4(A, l0, l1, l2, l3);
    else acc_add4(A, l0, l1, l2, l3);
}

__host__ __device__ __forceinline__ unsigned long long mulhi64(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

// Adds the exact product x y.  flags |= 1 for a non-finite operand, 2 when
// the exponents allow a product of magnitude >= 2^30 (neither is added).
// Bits of the product below 2^-192 are dropped toward zero.
__host__ __device__ __forceinline__ void acc_add_product(Acc4& A, double x, double y, unsigned& flags) {
    const unsigned long long bx = dbits(x), by = dbits(y);
    int ex = (int)((bx >> 52) & 0x7FF), ey = (int)((by >> 52) & 0x7FF);
    if (ex == 0x7FF || ey == 0x7FF) {
        flags |= 1u;
        return;
    }
    unsigned long long mx = bx & 0x000FFFFFFFFFFFFFull, my = by & 0x000FFFFFFFFFFFFFull;
    if (ex) mx |= 1ull << 52; else ex = 1;
    if (ey) my |= 1ull << 52; else ey = 1;
    if (mx == 0 || my == 0) return;
    if (ex + ey > 2074) {   // |x| < 2^(ex-1022), |y| < 2^(ey-1022)
        flags |= 2u;
        return;
    }
    unsigned long long lo = mx * my, hi = mulhi64(mx, my);
    int s = ex + ey - 1958;   // accumulator bit of the product's lowest bit (<= 116)
    if (s < 0) {
        const int t = -s;
        if (t >= 128) return;
        if (t >= 64) { lo = hi >> (t - 64); hi = 0; }
        else { lo = (lo >> t) | (hi << (64 - t)); hi >>= t; }
        s = 0;
    }
    const int r = s & 63;
    const unsigned long long w0 = lo << r;
    const unsigned long long w1 = (hi << r) | (r ? lo >> (64 - r) : 0ull);
    const unsigned long long w2 = r ? hi >> (64 - r) : 0ull;
    const bool q1 = s >= 64;
    const unsigned long long l0 = q1 ? 0ull : w0, l1 = q1 ? w0 : w1, l2 = q1 ? w1 : w2, l3 = q1 ? w2 : 0ull;
    if ((bx ^ by) >> 63) acc_sub4(A, l0, l1, l2, l3);
    else acc_add4(A, l0, l1, l2, l3);
}

__device__ __forceinline__ void acc_shfl_down_add(Acc4& A, int o) {
    Acc4 B;
#pragma unroll
    for (int q = 0; q < 4; ++q) B.w[q] = __shfl_down_sync(0xffffffffu, A.w[q], o);
    acc_add(A, B);
}

__device__ __forceinline__ void acc_warp_sum(Acc4& A) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc_shfl_down_add(A, o);
}

// Bits [pos, pos + 64) of the 256-bit magnitude (zero beyond the top).
__host__ __device__ inline unsigned long long acc_bits64(const unsigned long long* w, int pos) {
    const int q = pos >> 6, r = pos & 63;
    const unsigned long long lo = q < 4 ? w[q] >> r : 0ull;
    const unsigned long long hi = (r && q + 1 < 4) ? (w[q + 1] << (64 - r)) : 0ull;
    return lo | hi;
}

// The total rounded to the nearest double, ties to even.
__host__ __device__ inline double acc_to_double(const Acc4& A) {
    unsigned long long w[4] = {A.w[0], A.w[1], A.w[2], A.w[3]};
    const bool neg = (w[3] >> 63) != 0;
    if (neg) {   // two's-complement negation
        unsigned long long carry = 1ull;
        for (int q = 0; q < 4; ++q) {
            w[q] = ~w[q] + carry;
            carry = (carry && w[q] == 0ull) ? 1ull : 0ull;
        }
    }
    int top = -1;
    for (int q = 3; q >= 0 && top < 0; --q) {
        if (w[q]) {
            int b = 63;
            while (!((w[q] >> b) & 1ull)) --b;
            top = 64 * q + b;
        }
    }
    if (top < 0) return 0.0;
    unsigned long long M;
    int lsb;   // position of M's lowest bit
    if (top <= 52) {
        M = w[0];
        lsb = 0;
    } else {
        lsb = top - 52;
        M = acc_bits64(w, lsb) & ((1ull << 53) - 1ull);
        const bool round = (acc_bits64(w, lsb - 1) & 1ull) != 0;
        bool sticky = false;
        for (int q = 0; q < 4 && !sticky; ++q) {
            const int lo = 64 * q;
            if (lo >= lsb - 1) break;
            const int nb = (lsb - 1 - lo) < 64 ? (lsb - 1 - lo) : 64;
            const unsigned long long mask = nb == 64 ? ~0ull : ((1ull << nb) - 1ull);
            sticky = (w[q] & mask) != 0ull;
        }
        if (round && (sticky || (M & 1ull))) {
            M += 1ull;
            if (M >> 53) {
                M >>= 1;
                lsb += 1;
            }
        }
    }
    // value = M * 2^(lsb - 192); M < 2^53, so the conversion is exact and the
    // power of two is within the normal range (2^-192 .. 2^63)
    double v = (double)M;
    int ex = lsb - 192;
    while (ex > 0) { v *= 2.0; --ex; }
    while (ex < 0) {
        const int st = ex < -60 ? 60 : -ex;
        v /= (double)(1ull << st);
        ex += st;
    }
    return neg ? -v : v;
}

// ---------------------------------------------------------------------------
// exact division by a fixed divisor
// ---------------------------------------------------------------------------

struct DivConst {
    double y;                 // the divisor
    double inv;               // 1/y when y is a power of two (then x/y == x*inv exactly)
    unsigned long long My;    // significand of y with its leading bit, in [2^52, 2^53)
    unsigned long long R;     // floor(2^116 / My) (My > 2^52)
    int ey;                   // biased exponent of y
    int mode;                 // 0: native division, 1: integer quotient, 2: power of two
};

inline DivConst make_div_const(double y) {
    DivConst D{};
    D.y = y;
    D.mode = 0;
    unsigned long long b;
    static_assert(sizeof b == sizeof y, "double is 64-bit");
    __builtin_memcpy(&b, &y, sizeof b);
    const int e = (int)((b >> 52) & 0x7FF);
    if ((b >> 63) || e == 0 || e == 0x7FF) return D;   // negative, zero, subnormal, inf, nan
    D.ey = e;
    D.My = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
    if (D.My == (1ull << 52)) {
        D.inv = 1.0 / y;
        D.mode = 2;
        return D;
    }
    const unsigned __int128 one = (unsigned __int128)1 << 116;
    D.R = (unsigned long long)(one / D.My);
    D.mode = 1;
    return D;
}

// RN(x / D.y), bit-equal to x / D.y for every x.
__host__ __device__ __forceinline__ double div_exact(double x, const DivConst& D) {
    if (D.mode == 2) return x * D.inv;
    if (D.mode == 0) return x / D.y;
    const unsigned long long bx = dbits(x);
    const int ex = (int)((bx >> 52) & 0x7FF);
    if (ex == 0 || ex == 0x7FF) return x / D.y;
    const unsigned long long mx = (bx & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
    const bool ge = mx >= D.My;
    const int sh = ge ? 52 : 53;
    const unsigned long long lo = mx * D.R;
    const unsigned long long hi = mulhi64(mx, D.R);
    // floor(mx R / 2^(116 - sh)): the quotient or one less
    unsigned long long Q = ge ? hi : ((hi << 1) | (lo >> 63));
    unsigned long long rem = (mx << sh) - Q * D.My;   // exact: the true remainder is below 2 My < 2^54
    if (rem >= D.My) {
        Q += 1ull;
        rem -= D.My;
    }
    const unsigned long long twice = rem << 1;
    if (twice > D.My || (twice == D.My && (Q & 1ull))) Q += 1ull;
    int E = ex - D.ey - sh + 1075;
    if (Q >> 53) {   // rounded up to 2^53
        Q >>= 1;
        E += 1;
    }
    if (E <= 0 || E >= 0x7FF) return x / D.y;   // subnormal or infinite quotient
    return bitsd((bx & 0x8000000000000000ull) | ((unsigned long long)E << 52) | (Q & 0x000FFFFFFFFFFFFFull));
}

}  // namespace iegpu
