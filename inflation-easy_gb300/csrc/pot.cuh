// pot.cuh -- potential evaluation shared by the leapfrog, deltaN and
// reduction kernels.
//
// Hilltop (src/potential.cpp:77-83):
//   V  = V0 (1 - c1 v^2) / B^2,  c1 = (1 - ns)/4
//   V' = (c2 v) / B^2,           c2 = -V0 (1 - ns)/2
// The division by B^2 is the correctly rounded quotient formed on the integer
// pipes (div_exact, exact.cuh), bit-equal to the IEEE division.
// Tabulated (src/potential.cpp:11-68): the bracket l is the unique index with
// x[l-1] >= v > x[l] on the descending table, so the reference's hinted walk
// and its binary search agree; here a binary search over monotone 64-bit
// integer keys of the nodes finds it without FP64 compares.  Interpolation
// keeps the reference's expression y1 + ((v - x1)(y0 - y1))/(x0 - x1), with
// the differences y0 - y1 and x0 - x1 precomputed per bracket (the same IEEE
// values the reference computes on each call).
#pragma once
#include "iegpu_internal.cuh"

namespace iegpu {

// Monotone map from doubles to signed 64-bit integers (-0 folded onto +0).
__host__ __device__ inline long long order_key(double v) {
    v = v + 0.0;
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(v);
#else
    long long b;
    memcpy(&b, &v, sizeof b);
#endif
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}

__device__ __forceinline__ bool is_nan_bits(double v) {
    const long long b = __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFLL;
    return b > 0x7FF0000000000000LL;
}

// Bracket index and range flag (src/potential.cpp:19-38), from the n
// monotone keys of the descending nodes.
__device__ __forceinline__ int table_bracket_keys(const long long* key, int n, double v, bool* out_of_range) {
    const long long kv = order_key(v);
    const bool nan = is_nan_bits(v);
    *out_of_range = !nan && (kv > __ldg(&key[0]) || kv < __ldg(&key[n - 1]));
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = lo + ((hi - lo) >> 1);
        if (__ldg(&key[mid]) >= kv) lo = mid;
        else hi = mid;
    }
    return hi;
}

__device__ __forceinline__ int table_bracket(const PotDev& P, double v, bool* out_of_range) {
    return table_bracket_keys(P.key, P.n, v, out_of_range);
}

// Hinted bracket for a slowly moving value (deltaN loop): walks from l.
__device__ __forceinline__ int table_walk(const PotDev& P, double v, int l, bool* out_of_range) {
    const long long kv = order_key(v);
    const bool nan = is_nan_bits(v);
    const int n = P.n;
    *out_of_range = !nan && (kv > __ldg(&P.key[0]) || kv < __ldg(&P.key[n - 1]));
    if (nan || *out_of_range) return table_bracket(P, v, out_of_range);
    l = l < 1 ? 1 : (l > n - 1 ? n - 1 : l);
    while (l < n - 1 && __ldg(&P.key[l]) >= kv) ++l;
    while (l > 1 && __ldg(&P.key[l - 1]) < kv) --l;
    return l;
}

// interpolate_from_table, src/potential.cpp:52-68; the division by the
// bracket width x[l-1] - x[l] uses the bracket's precomputed divisor (exact).
__device__ __forceinline__ double table_interp(const PotDev& P, const double* y, const double* dy, double v, int l) {
    return __ldg(&y[l]) + div_exact((v - __ldg(&P.x[l])) * __ldg(&dy[l]), P.ddx[l]);
}

// potential_derivative at one site (src/potential.cpp:103-112), exact form.
template <bool TABLE>
__device__ __forceinline__ double dV_exact(const PotDev& P, double v, bool* oor) {
    if (TABLE) {
        const int l = table_bracket(P, v, oor);
        return div_exact(table_interp(P, P.dV, P.dydV, v, l), P.divB2);
    }
    *oor = false;
    return div_exact(P.c2 * v, P.divB2);
}

// potential(v) (src/potential.cpp:91-98), exact form.
template <bool TABLE>
__device__ __forceinline__ double V_exact(const PotDev& P, double v, bool* oor) {
    if (TABLE) {
        const int l = table_bracket(P, v, oor);
        return div_exact(table_interp(P, P.V, P.dyV, v, l), P.divB2);
    }
    *oor = false;
    return div_exact(P.V0 * (1.0 - P.c1 * (v * v)), P.divB2);
}

// Table value of V for the lattice-mean reduction (times B^2, no divide):
// the sum is re-associated anyway, so the slope form is used.
__device__ __forceinline__ double V_table_sum_term(const PotDev& P, double v, bool* oor) {
    const int l = table_bracket(P, v, oor);
    return __ldg(&P.V[l]) + (v - __ldg(&P.x[l])) * __ldg(&P.slopeV[l]);
}

__device__ __forceinline__ void flag_error(DevCtl* ctl, int code, double val) {
    if (atomicCAS(&ctl->error, 0, code) == 0) ctl->errval = val;
}

}  // namespace iegpu
