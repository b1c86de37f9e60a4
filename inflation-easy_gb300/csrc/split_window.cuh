// split_window.cuh -- brackets of a table window around a background
// value: the bracket search over the window and the register cache of the
// brackets nearest the background, used per site by the split step kernels.
// Host and device code, so that tests/native/window_cache_check.cu checks the
// caches against a search over the whole window on the CPU.
#pragma once

#include "iegpu_internal.cuh"

namespace iegpu {

// ---------------------------------------------------------------------------
// windows of table brackets around a background value
// ---------------------------------------------------------------------------

// Bracket q of the window with u[q+1] < v <= u[q]; -1 outside the window.
// The window is centred on the background value and a perturbation is a
// small fraction of a bracket, so a walk from the middle bracket ends after
// one or two compares (u descends strictly, so the bracket is unique).
__host__ __device__ __forceinline__ int window_find(const float* u, int n, float v) {
    if (!(v <= u[0] && v > u[n])) return -1;
    int q = n >> 1;
    while (v > u[q]) --q;
    while (v <= u[q + 1]) ++q;
    return q;
}

// The same bracket without branches, for lattices whose perturbations span
// several brackets (512^3: 1 % of the sites lie beyond the background's
// bracket and its neighbours, enough for divergent walks in a quarter of the
// warps to cost more than the search): the brackets with
// u[q] >= v form a prefix of the descending nodes (n + 1 of them, n <= kWin
// < 32) and q is its last index, found by binary lifting over the node
// indices with one shared-memory load per step.
__host__ __device__ __forceinline__ int window_lift(const float* u, int n, float v) {
    int q = 0;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int st = 16; st > 0; st >>= 1) {
        const int jn = q + st;
        const float uj = u[jn < n ? jn : n];
        q = (jn < n && uj >= v) ? jn : q;
    }
    return (v <= u[0] && v > u[n]) ? q : -1;
}

// The window's bracket of the background value (dphi = 0) and its two
// neighbours, bounds and lines kept in registers.  Perturbations are a small
// fraction of a bracket, so nearly every site falls in one of the three, which
// is chosen by selects without a branch (a warp's lanes do not diverge when a
// few of its sites lie in a neighbour).  Only a site beyond the neighbours
// searches the window.  Any of these finds the same bracket, which is unique.
// The wide cache (WIDE) also holds the brackets two away, for lattices whose
// perturbations reach them (512^3: about 1 % of the sites lie beyond the
// neighbours, so a quarter of a warp's lookups would otherwise search); it
// chooses among five brackets with four more selects per coefficient and
// gives the same bracket, hence the same bits.
struct WinCache {
    float hi, lo, A, s;   // bracket q: lo < v <= hi, value A + s v
    float hi2, lo2;       // u[q-1] and u[q+2] (hi and lo when there is no such neighbour)
    float Al, sl, Ar, sr; // lines of brackets q-1 and q+1 (q's own when there is no such neighbour)
    float hi3, lo3;       // wide: u[q-2] and u[q+3] (hi2 and lo2 when there is no such bracket)
    float All, sll, Arr, srr;   // wide: lines of brackets q-2 and q+2
};

template <bool TABLE, bool WIDE = false>
__host__ __device__ __forceinline__ WinCache win_cache(const float* w, int n) {
    // empty interval
    WinCache c{-1.f, 1.f, 0.f, 0.f, -1.f, 1.f, 0.f, 0.f, 0.f, 0.f, -1.f, 1.f, 0.f, 0.f, 0.f, 0.f};
    if (TABLE) {
        const int q = window_find(w, n, 0.f);
        if (q >= 0) {
            const int ql = q > 0 ? q - 1 : q, qr = q + 1 < n ? q + 1 : q;
            c.hi = w[q];
            c.lo = w[q + 1];
            c.A = w[kWin + 1 + q];
            c.s = w[2 * kWin + 1 + q];
            c.hi2 = q > 0 ? w[q - 1] : w[q];
            c.lo2 = q + 2 <= n ? w[q + 2] : w[q + 1];
            c.Al = w[kWin + 1 + ql];
            c.sl = w[2 * kWin + 1 + ql];
            c.Ar = w[kWin + 1 + qr];
            c.sr = w[2 * kWin + 1 + qr];
            if (WIDE) {
                const int qll = q > 1 ? q - 2 : ql, qrr = q + 2 < n ? q + 2 : qr;
                c.hi3 = q > 1 ? w[q - 2] : c.hi2;
                c.lo3 = q + 3 <= n ? w[q + 3] : c.lo2;
                c.All = w[kWin + 1 + qll];
                c.sll = w[2 * kWin + 1 + qll];
                c.Arr = w[kWin + 1 + qrr];
                c.srr = w[2 * kWin + 1 + qrr];
            }
        }
    }
    return c;
}

// The line (A, s) of x from the cache, when x lies in one of its brackets
// (returns false otherwise).  Nested bounds: x > hi2 implies x > hi, and
// x <= lo2 implies x <= lo, so the later selects override the earlier.
template <bool WIDE>
__host__ __device__ __forceinline__ bool cache_line(const WinCache& c, float x, float& A, float& s) {
    if (WIDE) {
        if (!(x <= c.hi3 && x > c.lo3)) return false;
        const bool u1 = x > c.hi, u2 = x > c.hi2, d1 = x <= c.lo, d2 = x <= c.lo2;
        A = u1 ? c.Al : c.A;
        s = u1 ? c.sl : c.s;
        A = u2 ? c.All : A;
        s = u2 ? c.sll : s;
        A = d1 ? c.Ar : A;
        s = d1 ? c.sr : s;
        A = d2 ? c.Arr : A;
        s = d2 ? c.srr : s;
        return true;
    }
    if (!(x <= c.hi2 && x > c.lo2)) return false;
    A = x > c.hi ? c.Al : (x <= c.lo ? c.Ar : c.A);
    s = x > c.hi ? c.sl : (x <= c.lo ? c.sr : c.s);
    return true;
}

}  // namespace iegpu
