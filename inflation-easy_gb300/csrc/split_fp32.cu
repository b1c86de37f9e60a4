// split_fp32.cu -- the split-precision form of the leapfrog.
//
// The field is stored as phi = phibar(t) + dphi(x), phi' = pibar(t) + dpi(x):
// the homogeneous background (phibar, pibar) and the scale factor in FP64, the
// perturbations dphi, dpi (and h_ij) in FP32.  In exact arithmetic this is the
// reference's leapfrog (src/evolution.cpp:150-284) written for the two parts:
//   pibar' = pibar + d(-friction pibar - potnorm V'(phibar))
//   dpi'   = dpi + d(laplnorm lapl(dphi) - friction dpi - potnorm [V'(phibar+dphi) - V'(phibar)])
//   phibar' = phibar + d pibar',  dphi' = dphi + d dpi'
// The potential difference is exact for the hilltop (V' linear); for the
// tabulated potential each bracket l is a line, so V'(phibar+dphi) - V'(phibar)
// = A_l + s_l dphi with A_l, s_l formed in FP64 once per step for a window of
// brackets around phibar.
//
// One kernel per step.  Each CTA owns a TJ x TK tile of (j, k) columns and
// marches along i through a chunk of planes, keeping three planes of dphi in
// shared memory.  Besides the tile it recomputes the step on a one-cell halo
// on the +j and +k sides, which gives the new dphi on every forward
// neighbour, so the same pass also accumulates the sums the next step's
// Friedmann update needs: sum (dphi(x+e) - dphi(x))^2 (= -sum dphi lapl dphi,
// the gradient energy), sum dphi and sum dphi^2 (hilltop potential) or sum of
// V differences (table).  Sums are Kahan-compensated in FP32 per thread and
// combined in FP64.  The last CTA to finish runs the FP64 Friedmann and
// background update for the next step.  HBM traffic per site-update:
// read dphi, dpi; write dphi, dpi = 16 B (ping-pong buffers), halos from L2.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <vector>

#include "split_kernels.cuh"
#include "split_rows4.cuh"

namespace iegpu {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// The sums of the current dphi at the start of a leapfrog call, all CTAs of one lattice.
template <bool TABLE>
__global__ void __launch_bounds__(kThreads) k_split_prime(const float* __restrict__ x, SplitCtl* ctl, PotDev P,
                                                          SplitConst K, double* part, unsigned* counter,
                                                          double* a_trace, int lg) {
    prime_body<TABLE>(x, ctl, P, K, part, counter, a_trace, lg, blockIdx.x + gridDim.x * blockIdx.y,
                      gridDim.x * gridDim.y, nullptr);
}

// The fused step.  Block (tile, chunk); TK = tile width along k (warp lanes).
// Shared rows hold k = -1 .. TK+1 at columns kColOff-1 .. kColOff+TK+1 with
// the tile interior 16-byte aligned, so each interior row segment arrives as
// TK/4 16-byte copies and the three halo columns as 4-byte copies.
template <bool TABLE, int TK>
__global__ void __launch_bounds__(256, 4) k_split_step(SplitBufs B, SplitCtl* ctl, PotDev P, SplitConst K, double* part,
                                                    unsigned* counter, double* a_trace, int lg, int TJ, int CH) {
    extern __shared__ __align__(16) float smem[];
    const int N = 1 << lg, m = N - 1;
    constexpr int RS = TK + 8;             // row stride (floats, multiple of 4)
    const int RP = (TJ + 3) * RS;          // dphi plane: rows j = -1 .. TJ+1
    const int PP = (TJ + 1) * RS;          // dpi plane: rows j = 0 .. TJ
    const int NS = TK + 1;                 // new-plane row stride (k from 0 .. TK)
    const int NP = (TJ + 1) * NS;          // new-plane size
    float* ring = smem;                    // kPhiSlots dphi planes
    float* pis = ring + kPhiSlots * RP;    // kPiSlots dpi planes
    float* nw = pis + kPiSlots * PP;       // 2 planes of new dphi
    float* wk = nw + 2 * NP;               // kick window: u[kWin+1], A[kWin], s[kWin]
    float* wv = wk + 3 * kWin + 1;         // potential window
    __shared__ int nk_s, nv_s, active_s;
    __shared__ double wbar[4];
    __shared__ float cf[6];
    const int tid = threadIdx.x, nthr = blockDim.x;
    if (tid == 0) {
        const SplitCtl& C = *ctl;
        active_s = C.active;
        cf[0] = C.d; cf[1] = C.lapl; cf[2] = C.fric; cf[3] = C.pn; cf[4] = C.kv;
        nk_s = C.wk.n;
        nv_s = C.wv.n;
    }
    if (TABLE) {
        for (int q = tid; q <= kWin; q += nthr) { wk[q] = ctl->wk.u[q]; wv[q] = ctl->wv.u[q]; }
        for (int q = tid; q < kWin; q += nthr) {
            wk[kWin + 1 + q] = ctl->wk.A[q]; wk[2 * kWin + 1 + q] = ctl->wk.s[q];
            wv[kWin + 1 + q] = ctl->wv.A[q]; wv[2 * kWin + 1 + q] = ctl->wv.s[q];
        }
        load_win_centres<false>(wbar, ctl);
    }
    __syncthreads();
    if (!active_s) return;
    const float d = cf[0], lap_n = cf[1], fric = cf[2], pn = cf[3], kv = cf[4];
    const WinCache ck = win_cache<TABLE>(wk, nk_s), cv = win_cache<TABLE>(wv, nv_s);
    const int ntj = N / TJ;
    const int tj = blockIdx.x % ntj, tk = blockIdx.x / ntj;
    const int j0 = tj * TJ, k0 = tk * TK, i0 = blockIdx.y * CH;
    const int cells = (TJ + 1) * (TK + 1);
    constexpr int QV = TK / 4;             // 16-byte segments per interior row

    // dphi plane i (rows j0-1 .. j0+TJ+1, columns k0-1 .. k0+TK+1)
    auto issue_phi = [&](int i) {
        float* dst = ring + ((i - i0 + 1) % kPhiSlots) * RP;
        const float* src = B.xs + ((long long)(i & m) << (2 * lg));
        const int ops = (TJ + 3) * (QV + 3);
        for (int o = tid; o < ops; o += nthr) {
            const int r = o / (QV + 3), w = o - r * (QV + 3);
            const float* row = src + ((long long)((j0 + r - 1) & m) << lg);
            float* srow = dst + r * RS;
            if (w < QV) cp_async16(srow + kColOff + 4 * w, row + k0 + 4 * w);
            else {
                const int kl = (w == QV) ? -1 : TK + (w - QV - 1);
                cp_async4(srow + kColOff + kl, row + ((k0 + kl) & m));
            }
        }
    };
    // dpi plane i (rows j0 .. j0+TJ, columns k0 .. k0+TK)
    auto issue_pi = [&](int i) {
        float* dst = pis + ((i - i0) % kPiSlots) * PP;
        const float* src = B.ps + ((long long)(i & m) << (2 * lg));
        const int ops = (TJ + 1) * (QV + 1);
        for (int o = tid; o < ops; o += nthr) {
            const int r = o / (QV + 1), w = o - r * (QV + 1);
            const float* row = src + ((long long)((j0 + r) & m) << lg);
            float* srow = dst + r * RS;
            if (w < QV) cp_async16(srow + kColOff + 4 * w, row + k0 + 4 * w);
            else cp_async4(srow + kColOff + TK, row + ((k0 + TK) & m));
        }
    };

    Kahan g, s1, s2;
    bool bad = false;
    issue_phi(i0 - 1);
    issue_phi(i0);
    cp_commit();
    for (int q = 0; q < kPrefetch; ++q) {
        if (q + 1 <= CH + 1) issue_phi(i0 + 1 + q);
        if (q <= CH) issue_pi(i0 + q);
        cp_commit();
    }
    for (int p = 0; p <= CH; ++p) {
        const int i = i0 + p;
        cp_wait<kPrefetch - 1>();
        __syncthreads();
        const float* pc = ring + ((p + 1) % kPhiSlots) * RP;
        const float* pu = ring + ((p + 2) % kPhiSlots) * RP;
        const float* pl = ring + (p % kPhiSlots) * RP;
        const float* pp = pis + (p % kPiSlots) * PP;
        float* nc = nw + (p & 1) * NP;
        const long long pb = (long long)(i & m) << (2 * lg);
        for (int cix = tid; cix < cells; cix += nthr) {
            int jl, kl;
            if (cix < TJ * TK) { jl = cix / TK; kl = cix - jl * TK; }
            else {
                const int h = cix - TJ * TK;
                if (h <= TK) { jl = TJ; kl = h; }
                else { jl = h - (TK + 1); kl = TK; }
            }
            const int o = (jl + 1) * RS + (kl + kColOff);
            const float x = pc[o];
            const float lap = pc[o + 1] + pc[o - 1] + pc[o + RS] + pc[o - RS] + pu[o] + pl[o] - 6.f * x;
            const float pi0 = pp[jl * RS + kl + kColOff];
            const float dv = split_dv<TABLE>(x, wk, nk_s, ck, pn, kv, bad, P, wbar);
            const float pin = pi0 + d * (lap_n * lap - fric * pi0 - dv);
            const float xn = x + d * pin;
            nc[jl * NS + kl] = xn;
            if (jl < TJ && kl < TK && p < CH) {
                const long long gi = pb + ((long long)(j0 + jl) << lg) + (k0 + kl);
                B.xd[gi] = xn;
                B.pd[gi] = pin;
                s1.add(xn);
                const float v2 = split_v<TABLE>(xn, wv, nv_s, cv, bad, P, wbar + 2);
                if (!TABLE || !bad) s2.add(v2);
            }
        }
        __syncthreads();
        // planes kPrefetch ahead (the slots of planes no longer needed)
        if (p + kPrefetch + 1 <= CH + 1) issue_phi(i + 1 + kPrefetch);
        if (p + kPrefetch <= CH) issue_pi(i + kPrefetch);
        cp_commit();
        const float* np_ = nw + ((p + 1) & 1) * NP;  // previous plane's new values
        for (int cix = tid; cix < TJ * TK; cix += nthr) {
            const int jl = cix / TK, kl = cix - jl * TK;
            const float xc = nc[jl * NS + kl];
            if (p < CH) {
                const float dk = nc[jl * NS + kl + 1] - xc;
                const float dj = nc[(jl + 1) * NS + kl] - xc;
                g.add(dk * dk + dj * dj);
            }
            if (p >= 1) {
                const float di = xc - np_[jl * NS + kl];
                g.add(di * di);
            }
        }
    }
    cp_wait<0>();
    if (bad) {
        if (atomicCAS(&ctl->error, 0, IEGPU_ERANGE) == 0) ctl->errval = ctl->phibar;
    }
    maybe_precompute(ctl, P, K);
    df64 v[3] = {g.df(), s1.df(), s2.df()};
    finish_sums(v, ctl, P, K, part, counter, a_trace);
}
template <bool TABLE, int C, int TJ, int PF>
__global__ void __launch_bounds__((TJ + 1) * 32) k_split_rows(SplitBufs B, SplitCtl* ctl, PotDev P, SplitConst K,
                                                              double* part, unsigned* counter, double* a_trace,
                                                              int chunks) {
    constexpr int N = 32 * C;
    pdl_begin();
    const int i0 = (int)(((long long)blockIdx.y * N) / chunks);
    const int CH = (int)(((long long)(blockIdx.y + 1) * N) / chunks) - i0;
    rows_body<TABLE, C, TJ, PF>(B, ctl, P, K, part, counter, a_trace, blockIdx.x * TJ, i0, CH,
                                blockIdx.x + gridDim.x * blockIdx.y, gridDim.x * gridDim.y, nullptr);
}


// Whole planes (N = 32, 64): block y = chunk of planes.
template <bool TABLE, int N, int NT, int PF>
__global__ void __launch_bounds__(NT, plane_min_ctas(N)) k_split_plane(SplitBufs B, SplitCtl* ctl, PotDev P, SplitConst K, double* part,
                                                    unsigned* counter, double* a_trace, int chunks) {
    pdl_begin();
    const int i0 = (int)(((long long)blockIdx.y * N) / chunks);
    const int CH = (int)(((long long)(blockIdx.y + 1) * N) / chunks) - i0;
    plane_body<TABLE, N, NT, PF>(B, ctl, P, K, part, counter, a_trace, i0, CH, blockIdx.x + gridDim.x * blockIdx.y,
                                 gridDim.x * gridDim.y, nullptr);
}

// SIGW in the split form: h kick and drift for the coming step, before the
// scalar step kernel replaces the coefficients (src/evolution.cpp:183-254,
// 272-281 with the source built from the FP32 dphi gradients).
__global__ void __launch_bounds__(kThreads) k_split_h(const float* __restrict__ x, SigwSplit S, const SplitCtl* ctl,
                                                      int lg, float half_over_dx, int kick_only) {
    const int active = ctl->active;
    if (!active) return;
    const float d = ctl->d, lap_n = ctl->lapl, fric = ctl->fric, src = ctl->srcAmp;
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    const int m = (1 << lg) - 1;
    const int k = (int)(id & m), j = (int)((id >> lg) & m), i = (int)(id >> (2 * lg));
    const long long kp = id - k + ((k + 1) & m), km = id - k + ((k - 1) & m);
    const long long jp = id + ((long long)(((j + 1) & m) - j) << lg), jm = id + ((long long)(((j - 1) & m) - j) << lg);
    const long long ip = id + ((long long)(((i + 1) & m) - i) << (2 * lg));
    const long long im = id + ((long long)(((i - 1) & m) - i) << (2 * lg));
    const float gx = (x[ip] - x[im]) * half_over_dx;
    const float gy = (x[jp] - x[jm]) * half_over_dx;
    const float gz = (x[kp] - x[km]) * half_over_dx;
    const float T[6] = {gx * gx, gy * gy, gz * gz, gx * gy, gx * gz, gy * gz};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const float* h = S.hs[c];
        const float hc = h[id];
        const float lf = h[kp] + h[km] + h[jp] + h[jm] + h[ip] + h[im] - 6.f * hc;
        const float hdo = S.hd[c][id];
        const float hdn = hdo + d * (lap_n * lf - fric * hdo + src * T[c]);
        S.hd[c][id] = hdn;
        if (!kick_only) S.hdst[c][id] = hc + d * hdn;
    }
}

// The same update with each thread on four consecutive sites along k:
// 128-bit loads of the centre, j +- 1, i +- 1 values and of h', two scalar
// loads for k - 1 and k + 4 (periodic), and the arithmetic of k_split_h per
// site in the same order.
__global__ void __launch_bounds__(kThreads) k_split_h4(const float* __restrict__ x, SigwSplit S, const SplitCtl* ctl,
                                                       int lg, float half_over_dx, int kick_only) {
    const int active = ctl->active;
    if (!active) return;
    const float d = ctl->d, lap_n = ctl->lapl, fric = ctl->fric, src = ctl->srcAmp;
    const long long id = 4LL * ((long long)blockIdx.x * kThreads + threadIdx.x);
    const int m = (1 << lg) - 1;
    const int k = (int)(id & m), j = (int)((id >> lg) & m), i = (int)(id >> (2 * lg));
    const long long row = id - k;
    const long long km = row + ((k - 1) & m), k4 = row + ((k + 4) & m);
    const long long jp = id + ((long long)(((j + 1) & m) - j) << lg), jm = id + ((long long)(((j - 1) & m) - j) << lg);
    const long long ip = id + ((long long)(((i + 1) & m) - i) << (2 * lg));
    const long long im = id + ((long long)(((i - 1) & m) - i) << (2 * lg));
    auto ld4g = [](const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); };
    const float4 xc = ld4g(x + id), xjp = ld4g(x + jp), xjm = ld4g(x + jm), xip = ld4g(x + ip), xim = ld4g(x + im);
    const float xkm = __ldg(x + km), xk4 = __ldg(x + k4);
    const float xv[6] = {xkm, xc.x, xc.y, xc.z, xc.w, xk4};
    const float jpv[4] = {xjp.x, xjp.y, xjp.z, xjp.w}, jmv[4] = {xjm.x, xjm.y, xjm.z, xjm.w};
    const float ipv[4] = {xip.x, xip.y, xip.z, xip.w}, imv[4] = {xim.x, xim.y, xim.z, xim.w};
    float T[6][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const float gx = (ipv[e] - imv[e]) * half_over_dx;
        const float gy = (jpv[e] - jmv[e]) * half_over_dx;
        const float gz = (xv[e + 2] - xv[e]) * half_over_dx;
        T[0][e] = gx * gx; T[1][e] = gy * gy; T[2][e] = gz * gz;
        T[3][e] = gx * gy; T[4][e] = gx * gz; T[5][e] = gy * gz;
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const float* h = S.hs[c];
        const float4 hc4 = ld4g(h + id), hjp = ld4g(h + jp), hjm = ld4g(h + jm), hip = ld4g(h + ip), him = ld4g(h + im);
        const float hv[6] = {__ldg(h + km), hc4.x, hc4.y, hc4.z, hc4.w, __ldg(h + k4)};
        const float hjpv[4] = {hjp.x, hjp.y, hjp.z, hjp.w}, hjmv[4] = {hjm.x, hjm.y, hjm.z, hjm.w};
        const float hipv[4] = {hip.x, hip.y, hip.z, hip.w}, himv[4] = {him.x, him.y, him.z, him.w};
        const float4 hd4 = *reinterpret_cast<const float4*>(S.hd[c] + id);
        const float hdv[4] = {hd4.x, hd4.y, hd4.z, hd4.w};
        float hdn[4], hn[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float hc = hv[e + 1];
            const float lf = hv[e + 2] + hv[e] + hjpv[e] + hjmv[e] + hipv[e] + himv[e] - 6.f * hc;
            hdn[e] = hdv[e] + d * (lap_n * lf - fric * hdv[e] + src * T[c][e]);
            hn[e] = hc + d * hdn[e];
        }
        *reinterpret_cast<float4*>(S.hd[c] + id) = make_float4(hdn[0], hdn[1], hdn[2], hdn[3]);
        if (!kick_only) *reinterpret_cast<float4*>(S.hdst[c] + id) = make_float4(hn[0], hn[1], hn[2], hn[3]);
    }
}

// evolve_fields in the split form (in place): dphi += d dpi, h += d hd, and
// phibar += d pibar for the background.
__global__ void k_split_drift(float* __restrict__ x, const float* __restrict__ p, SigwSplit S, int sigw, long long gs,
                              double d, SplitCtl* ctl) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id == 0) ctl->phibar = ctl->phibar + d * ctl->pibar;
    if (id >= gs) return;
    const float df = (float)d;
    x[id] = x[id] + df * p[id];
    if (sigw) {
#pragma unroll
        for (int c = 0; c < 6; ++c) S.hdst[c][id] = S.hdst[c][id] + df * S.hd[c][id];
    }
}

// Kick only (evolve_derivs): dpi += d(...) with the current coefficients.
template <bool TABLE>
__global__ void __launch_bounds__(kThreads) k_split_kick(const float* __restrict__ x, float* __restrict__ p,
                                                         SplitCtl* ctl, PotDev P, int lg) {
    __shared__ float wk[3 * kWin + 1];
    __shared__ double wbar[4];
    __shared__ int nk;
    if (!ctl->active) return;
    if (TABLE) {
        for (int q = threadIdx.x; q <= kWin; q += blockDim.x) wk[q] = ctl->wk.u[q];
        for (int q = threadIdx.x; q < kWin; q += blockDim.x) { wk[kWin + 1 + q] = ctl->wk.A[q]; wk[2 * kWin + 1 + q] = ctl->wk.s[q]; }
        if (threadIdx.x == 0) nk = ctl->wk.n;
        load_win_centres<false>(wbar, ctl);
        __syncthreads();
    }
    const float d = ctl->d, lap_n = ctl->lapl, fric = ctl->fric, pn = ctl->pn, kv = ctl->kv;
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    const int m = (1 << lg) - 1;
    const int k = (int)(id & m), j = (int)((id >> lg) & m), i = (int)(id >> (2 * lg));
    const float xc = x[id];
    const float lap = x[id - k + ((k + 1) & m)] + x[id - k + ((k - 1) & m)] +
                      x[id + ((long long)(((j + 1) & m) - j) << lg)] + x[id + ((long long)(((j - 1) & m) - j) << lg)] +
                      x[id + ((long long)(((i + 1) & m) - i) << (2 * lg))] +
                      x[id + ((long long)(((i - 1) & m) - i) << (2 * lg))] - 6.f * xc;
    float dv;
    bool bad = false;
    if (TABLE) {
        const int q = window_find(wk, nk, xc);
        dv = pn * (q < 0 ? far_line(P, P.dV, P.slopedV, wbar, xc, bad) : wk[kWin + 1 + q] + wk[2 * kWin + 1 + q] * xc);
    } else {
        dv = kv * xc;
    }
    const float p0 = p[id];
    p[id] = p0 + d * (lap_n * lap - fric * p0 - dv);
    if (TABLE && bad && atomicCAS(&ctl->error, 0, IEGPU_ERANGE) == 0) ctl->errval = (double)xc + wbar[0];
}

// residual of the compensated form as a double (0 without one)
__device__ __forceinline__ double residual(const unsigned short* r, long long id) {
    return r ? (double)__uint_as_float((unsigned)r[id] << 16) : 0.0;
}

// f64 = bar + (double)x (- residual)  (materialise the full field)
__global__ void k_split_materialize(const float* __restrict__ x, const unsigned short* __restrict__ res,
                                    double* __restrict__ out, long long gs, const SplitCtl* ctl, int which) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= gs) return;
    const double bar = which ? ctl->pibar : ctl->phibar;
    out[id] = bar + ((double)x[id] - residual(res, id));
}

// x = (float)(in - bar) with bar = mean of in (given)
__global__ void k_split_absorb(const double* __restrict__ in, float* __restrict__ x, long long gs, double bar) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= gs) return;
    x[id] = (float)(in[id] - bar);
}

// (double) x (- residual) for spectra of the perturbation
__global__ void k_split_to_double(const float* __restrict__ x, const unsigned short* __restrict__ res,
                                  double* __restrict__ out, long long gs) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id < gs) out[id] = (double)x[id] - residual(res, id);
}

// Lattice sums of the split state for energies / means:
// [0] sum dphi, [1] sum dphi^2, [2] sum dpi, [3] sum dpi^2, [4] sum sq forward diffs, [5] sum dV (table units)
template <bool TABLE>
__global__ void __launch_bounds__(kThreads) k_split_sums(const float* __restrict__ x, const float* __restrict__ p,
                                                         const SplitCtl* ctl, PotDev P, double* part, int lg) {
    __shared__ float su[kWin + 1], sA[kWin], ss[kWin];
    __shared__ double wb[2];
    __shared__ int sn;
    if (TABLE && threadIdx.x == 0) {
        SplitWin W;
        int err = 0;
        build_window(W, P, P.V, P.dyV, ctl->phibar, &err);
        sn = err ? -1 : W.n;
        wb[0] = W.phibar;
        wb[1] = W.Fbar;
        for (int q = 0; q <= W.n && !err; ++q) su[q] = W.u[q];
        for (int q = 0; q < W.n && !err; ++q) { sA[q] = W.A[q]; ss[q] = W.s[q]; }
    }
    __syncthreads();
    const long long gs = 1LL << (3 * lg);
    const int m = (1 << lg) - 1;
    Kahan a0, a1, a2, a3, a4, a5;
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const int k = (int)(id & m), j = (int)((id >> lg) & m), i = (int)(id >> (2 * lg));
        const float xc = x[id];
        const float dk = x[id - k + ((k + 1) & m)] - xc;
        const float dj = x[id + ((long long)(((j + 1) & m) - j) << lg)] - xc;
        const float di = x[id + ((long long)(((i + 1) & m) - i) << (2 * lg))] - xc;
        const float pc = p[id];
        a0.add(xc);
        a1.add(xc * xc);
        a2.add(pc);
        a3.add(pc * pc);
        a4.add(dk * dk + dj * dj + di * di);
        if (TABLE && sn >= 0) {
            const int q = window_find(su, sn, xc);
            bool bad = false;
            a5.add(q >= 0 ? sA[q] + ss[q] * xc : far_line(P, P.V, P.slopeV, wb, xc, bad));
        }
    }
    double v[6] = {a0.value(), a1.value(), a2.value(), a3.value(), a4.value(), a5.value()};
    block_sum<6>(v);
    if (threadIdx.x == 0)
        for (int q = 0; q < 6; ++q) part[6 * blockIdx.x + q] = v[q];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// chunks == 0 (N >= 128): one wave of CTAs, each with an equal share of the
// (row tile, plane) units, so every SM carries the same load.
static int balanced_ctas(const iegpu_ctx* c, int N, int TJ, int PF);

// Shared memory one row-kernel CTA needs, and how many fit on an SM.  TJ = N
// (N <= 64) selects the whole-plane kernel.
static bool plane_shape(int N, int TJ) { return TJ == N && (N == 32 || N == 64); }
static int plane_threads(int N) { return plane_nt(N); }

static size_t row_smem_bytes(int N, int TJ, int PF) {
    if (plane_shape(N, TJ)) return sizeof(float) * (size_t)split_plane_smem_floats(N, PF);
    return sizeof(float) * (size_t)(N >= 128 ? split_row4_smem_floats(TJ, N, PF) : split_row_smem_floats(TJ, N, PF));
}

static int row_ctas_per_sm(int N, int TJ, int PF) {
    const size_t smem = row_smem_bytes(N, TJ, PF) + 1024;
    const size_t per_sm = 228 * 1024;
    int by_smem = (int)(per_sm / smem);
    const int nthr = plane_shape(N, TJ) ? plane_threads(N) : N >= 128 ? row4_threads(TJ) : (TJ + 1) * 32;
    const int by_regs = 65536 / (nthr * 72);
    int n = by_smem < by_regs ? by_smem : by_regs;
    return n < 1 ? (smem <= 227 * 1024 ? 1 : 0) : n;
}

static int balanced_ctas(const iegpu_ctx* c, int N, int TJ, int PF) {
    const int per_sm = row_ctas_per_sm(N, TJ, PF);
    const long long units = (long long)(N / TJ) * N;
    long long n = (long long)c->sms * (per_sm > 0 ? per_sm : 1);
    return (int)(n < units ? n : units);
}

// Untuned choice: 8-row tiles (4 at N = 512), two planes prefetched, and a
// chunk count that makes the grid one wave of resident CTAs.
static RowCfg default_row_cfg(const iegpu_ctx* c) {
    RowCfg r;
    const int N = c->N;
    r.TJ = N >= 512 ? 4 : 8;
    r.PF = 2;   // also a compensated shape
    const int per_sm = row_ctas_per_sm(N, r.TJ, r.PF);
    const int tiles = N / r.TJ;
    int chunks = (c->sms * (per_sm > 0 ? per_sm : 1)) / tiles;
    if (chunks < 1) chunks = 1;
    if (chunks > N / 8) chunks = N / 8 > 0 ? N / 8 : 1;
    r.chunks = chunks;
    return r;
}

static StepGeom step_geom(const iegpu_ctx* c) {
    StepGeom g;
    const int N = c->N;
    if (N >= 32 && N <= 512) {
        g.rows = true;
        g.TK = N;
        RowCfg rc = c->row_cfg;
        if (rc.TJ == 0) rc = default_row_cfg(c);
        g.TJ = rc.TJ;
        g.PF = rc.PF;
        g.tma = rc.tma;
        g.chunks = rc.chunks;
        g.tiles = rc.chunks > 0 ? N / g.TJ : balanced_ctas(c, N, g.TJ, g.PF);
        g.CH = rc.chunks > 0 ? N / rc.chunks : 0;
        g.smem = row_smem_bytes(N, g.TJ, g.PF);
        return g;
    }
    g.rows = false;
    g.TK = N >= 32 ? 32 : N;
    g.TJ = 256 / g.TK;
    if (g.TJ > N) g.TJ = N;
    g.tiles = (N / g.TJ) * (N / g.TK);
    // one wave of resident CTAs (4 per SM at 64 registers); at least 8 planes per chunk
    int chunks = 1;
    while (chunks * 2 <= N / 8 && g.tiles * chunks * 2 <= c->sms * 4) chunks *= 2;
    g.chunks = chunks;
    g.CH = N / chunks;
    g.smem = sizeof(float) * (size_t)split_step_smem_floats(g.TJ, g.TK);
    return g;
}

static void launch_prime(iegpu_ctx* c, int src) {
    const SplitConst K = split_const(c);
    dim3 grid(c->red_grid, 1);
    if (c->pot.table)
        k_split_prime<true><<<grid, kThreads, 0, c->stream>>>(c->sp[src], c->sctl, c->pot, K, c->part, c->counter, c->a_trace, c->lg);
    else
        k_split_prime<false><<<grid, kThreads, 0, c->stream>>>(c->sp[src], c->sctl, c->pot, K, c->part, c->counter, c->a_trace, c->lg);
    c->launches++;
}

// Shapes of the compensated row kernel (instantiated for these alone): 16-row
// tiles (N <= 256) with 2 or 3 planes ahead, 8-row tiles with 2, 4-row tiles
// with 2 (N = 512); cp.async staging.
static bool comp_shape_ok(int N, int TJ, int PF, int tma) {
    if (tma || N < 128 || N > 512) return false;
    if (TJ == 16) return N <= 256 && (PF == 2 || PF == 3);
    if (TJ == 8) return PF == 2;
    return TJ == 4 && N == 512 && PF == 2;
}

static SigwSplit sigw_split(iegpu_ctx* c, int src) {
    SigwSplit S{};
    if (!c->cfg.sigw) return S;
    for (int q = 0; q < 6; ++q) {
        S.hs[q] = c->h[src][q];
        S.hdst[q] = c->h[src ^ 1][q];
        S.hd[q] = c->hd[q];
    }
    return S;
}

template <bool TAB, int CC, int TJV, int PFV>
static void rows_one(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    if (smem_optin((const void*)k_split_rows<TAB, CC, TJV, PFV>, g.smem) != cudaSuccess) {
        set_error(c, IEGPU_ECUDA, "shared memory opt-in of the split step kernel failed");   // the launch then fails
    }
    launch_pdl(k_split_rows<TAB, CC, TJV, PFV>, grid, dim3((TJV + 1) * 32), g.smem, c->stream, B, c->sctl, c->pot, K,
               c->part, c->counter, c->a_trace, g.chunks);
}

template <bool TAB, int NV, int PFV>
static void plane_one(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    constexpr int NT = plane_nt(NV);
    if (smem_optin((const void*)k_split_plane<TAB, NV, NT, PFV>, g.smem) != cudaSuccess) {
        set_error(c, IEGPU_ECUDA, "shared memory opt-in of the split step kernel failed");   // the launch then fails
    }
    launch_pdl(k_split_plane<TAB, NV, NT, PFV>, grid, dim3(NT), g.smem, c->stream, B, c->sctl, c->pot, K, c->part,
               c->counter, c->a_trace, g.chunks);
}

template <bool TAB, int NV>
static void plane_pf(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    if (g.PF == 4) plane_one<TAB, NV, 4>(c, B, K, grid, g);
    else plane_one<TAB, NV, 2>(c, B, K, grid, g);
}

template <bool TAB, int CC>
static void rows_tj(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    if (g.TJ == 4) { if (g.PF == 1) rows_one<TAB, CC, 4, 1>(c, B, K, grid, g); else rows_one<TAB, CC, 4, 2>(c, B, K, grid, g); }
    else { if (g.PF == 1) rows_one<TAB, CC, 8, 1>(c, B, K, grid, g); else rows_one<TAB, CC, 8, 2>(c, B, K, grid, g); }
}

template <bool TAB>
static void rows_c(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    switch (c->N) {
        case 32: if (g.TJ == 32) plane_pf<TAB, 32>(c, B, K, grid, g); else rows_tj<TAB, 1>(c, B, K, grid, g); break;
        case 64: if (g.TJ == 64) plane_pf<TAB, 64>(c, B, K, grid, g); else rows_tj<TAB, 2>(c, B, K, grid, g); break;
        case 128: rows4_launch_128(c, TAB, B, K, grid, g); break;
        case 256: rows4_launch_256(c, TAB, B, K, grid, g); break;
        default: rows4_launch_512(c, TAB, B, K, grid, g); break;
    }
}

static void launch_rows(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    if (c->pot.table) rows_c<true>(c, B, K, grid, g);
    else rows_c<false>(c, B, K, grid, g);
    c->launches++;
}

static void launch_step(iegpu_ctx* c, int src) {
    const SplitConst K = split_const(c);
    // the autotuner times the scalar step's shapes on a saved copy of dphi and
    // dpi alone: the tensors must not be stepped by its trial steps
    if (c->cfg.sigw && !c->tuning) {
        const float hodx = (float)(0.5 / K.dx);
        if (c->gs % (4 * kThreads) == 0)
            k_split_h4<<<(unsigned)(c->gs / (4 * kThreads)), kThreads, 0, c->stream>>>(c->sp[src], sigw_split(c, src),
                                                                                       c->sctl, c->lg, hodx, 0);
        else
            k_split_h<<<(unsigned)(c->gs / kThreads), kThreads, 0, c->stream>>>(c->sp[src], sigw_split(c, src), c->sctl,
                                                                                c->lg, hodx, 0);
        c->launches++;
    }
    StepGeom g = step_geom(c);
    g.rev = src & 1;
    const SplitBufs B = split_bufs(c, src);
    dim3 grid(g.tiles, g.chunks > 0 ? g.chunks : 1);
    if (g.rows) {
        launch_rows(c, B, K, grid, g);
        return;
    }
#define IEGPU_SPLIT_LAUNCH(TAB, TKV)                                                                          \
    k_split_step<TAB, TKV><<<grid, g.TJ * TKV, g.smem, c->stream>>>(B, c->sctl, c->pot, K, c->part, c->counter, \
                                                                    c->a_trace, c->lg, g.TJ, g.CH)
    const bool tab = c->pot.table != 0;
    if (g.TK == 32) { if (tab) IEGPU_SPLIT_LAUNCH(true, 32); else IEGPU_SPLIT_LAUNCH(false, 32); }
    else if (g.TK == 16) { if (tab) IEGPU_SPLIT_LAUNCH(true, 16); else IEGPU_SPLIT_LAUNCH(false, 16); }
    else { if (tab) IEGPU_SPLIT_LAUNCH(true, 8); else IEGPU_SPLIT_LAUNCH(false, 8); }
#undef IEGPU_SPLIT_LAUNCH
    c->launches++;
}

// ---- persistent launches (vector row kernel) ------------------------------

// 0: launched (or would launch, check_only); 1: this lattice steps kernel by
// kernel (persistent launches off, SIGW, N outside 128..256, bulk-copy
// staging, or a grid that is not resident at once); -1: launch error.
static int launch_persist(iegpu_ctx* c, int start, int nsteps, bool check_only) {
    // At N = 512 the step is long enough that the launch gap is noise, and the
    // persistent kernel measured slower (397 vs 378 us at 512^3).
    if (!c->persist || c->cfg.sigw || c->N < 128 || c->N > 256) return 1;
    const StepGeom g = step_geom(c);
    if (!g.rows || g.tma) return 1;
    const dim3 grid(g.tiles, g.chunks > 0 ? g.chunks : 1);
    const bool tab = c->pot.table != 0;
    switch (c->N) {
        case 128: return rows4_persist_128(c, tab, start, nsteps, grid, g, check_only);
        case 256: return rows4_persist_256(c, tab, start, nsteps, grid, g, check_only);
        case 512: return rows4_persist_512(c, tab, start, nsteps, grid, g, check_only);
        default: return 1;
    }
}

void split_destroy_graphs(iegpu_ctx* c) {
    for (int p = 0; p < 2; ++p) {
        if (c->sp_exec[p]) cudaGraphExecDestroy(c->sp_exec[p]);
        c->sp_exec[p] = nullptr;
    }
}

static int split_graph_steps(const iegpu_ctx* c) { return c->N <= 64 ? 32 : 8; }

static int split_build_graphs(iegpu_ctx* c) {
    const int L = split_graph_steps(c);
    for (int p = 0; p < 2; ++p) {
        cudaGraph_t gph;
        if (check_cuda(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "graph capture")) return IEGPU_ECUDA;
        const long long before = c->launches;
        for (int s = 0; s < L; ++s) launch_step(c, (p + s) & 1);
        c->launches = before;
        if (check_cuda(c, cudaStreamEndCapture(c->stream, &gph), "graph capture end")) return IEGPU_ECUDA;
        cudaError_t e = cudaGraphInstantiate(&c->sp_exec[p], gph, 0);
        cudaGraphDestroy(gph);
        if (check_cuda(c, e, "graph instantiate")) return IEGPU_ECUDA;
    }
    c->sp_steps = L;
    return IEGPU_OK;
}

static int sctl_up(iegpu_ctx* c) {
    return check_cuda(c, cudaMemcpyAsync(c->sctl, c->sctl_h, sizeof(SplitCtl), cudaMemcpyHostToDevice, c->stream), "split control upload");
}

static int sctl_down(iegpu_ctx* c) {
    if (check_cuda(c, cudaMemcpyAsync(c->sctl_h, c->sctl, sizeof(SplitCtl), cudaMemcpyDeviceToHost, c->stream), "split control download"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "split")) return IEGPU_ECUDA;
    // a wait that gave up ends the call's steps wherever they were, so a
    // deferred scalar update may be left over; the next call starts from the
    // host's copy of the background
    if (c->sctl_h->error == IEGPU_ETIMEOUT)
        return set_error(c, IEGPU_ETIMEOUT, "a wait in the step kernel gave up (bulk copy or step barrier)");
    if (c->sctl_h->deferred)
        return set_error(c, IEGPU_ECUDA, "internal: a scalar update was left unapplied at the end of a call");
    if (c->sctl_h->error == IEGPU_ERANGE) {
        return set_error(c, IEGPU_ERANGE,
                         "Field value near %.17g is outside the numerical potential range [%.17g, %.17g].\n",
                         c->sctl_h->errval, c->htab_x.empty() ? 0.0 : c->htab_x.back(),
                         c->htab_x.empty() ? 0.0 : c->htab_x.front());
    }
    return IEGPU_OK;
}

static void sctl_fill(iegpu_ctx* c, const iegpu_bg* bg, int mode) {
    SplitCtl& C = *c->sctl_h;
    C.bg.t = bg->t;
    C.bg.a = bg->a;
    C.bg.ad = bg->ad;
    C.bg.ad2 = bg->ad2;
    C.bg.astep = bg->astep;
    C.mode = mode;
    C.steps_done = 0;
    C.steps_limit = 0;
    C.done = 0;
    C.error = 0;
    C.active = 0;
    C.pre_claim = 0;
    C.pre.ok = 0;
    C.deferred = 0;
    C.spin_polls = c->wait_polls;
    C.spin_bias = c->wait_bias;
}

static void sctl_bg(const iegpu_ctx* c, iegpu_bg* bg) {
    const DevBg& B = c->sctl_h->bg;
    bg->t = B.t;
    bg->a = B.a;
    bg->ad = B.ad;
    bg->ad2 = B.ad2;
    bg->astep = B.astep;
}

int split_profile(iegpu_ctx* c, double af, int nsteps, iegpu_bg* bg, double* ms, int nk);
static int split_profile_persist(iegpu_ctx* c, int nsteps, iegpu_bg* bg, double* ms);

// Autotuner of the row kernel's launch shape: rows per tile (TJ), planes
// prefetched (PF) and plane chunks (grid height).  Each candidate runs one
// warm-up and three timed steps (CUDA events, stream-ordered) from a saved copy
// of dphi and dpi (and their residuals), which is restored afterwards; the
// trial steps do not step the tensors.  The fastest shape is kept for the
// life of the context.
static int split_autotune_shapes(iegpu_ctx* c, const iegpu_bg* bg0);

int split_autotune(iegpu_ctx* c, const iegpu_bg* bg0) {
    c->tuning = 1;
    const int rc = split_autotune_shapes(c, bg0);
    c->tuning = 0;
    return rc;
}

static int split_autotune_shapes(iegpu_ctx* c, const iegpu_bg* bg0) {
    const int N = c->N;
    c->tuned = 1;
    if (N < 32 || N > 512) return IEGPU_OK;
    std::vector<RowCfg> cands;
    if (N == 32 || N == 64) {
        // whole planes: N/8 .. N/32 chunks of planes
        for (int PF : {2, 4})
            for (int ch = N / 8; ch >= 1 && ch >= N / 32; ch /= 2)
                if (row_ctas_per_sm(N, N, PF) >= 1) {
                    RowCfg r;
                    r.TJ = N;
                    r.PF = PF;
                    r.chunks = ch;
                    cands.push_back(r);
                }
    }
    for (int TJ : {4, 8, 16}) {
        if (TJ > N || (TJ == 16 && (N < 128 || N > 256))) continue;
        for (int PF : {1, 2, 3, 4}) {
            if (PF > 2 && !((TJ == 4 && N >= 128) || (TJ == 16 && PF == 3))) continue;
            const int per_sm = row_ctas_per_sm(N, TJ, PF);
            if (per_sm < 1) continue;
            const int tiles = N / TJ;
            if (N >= 128) {
                RowCfg r;
                r.TJ = TJ;
                r.PF = PF;
                r.chunks = 0;   // balanced
                cands.push_back(r);
            }
            for (int waves : {1, 2}) {
                int ch = (waves * c->sms * per_sm) / tiles;
                if (ch < 1) ch = 1;
                if (ch > N / 8) ch = N / 8 > 0 ? N / 8 : 1;
                RowCfg r;
                r.TJ = TJ;
                r.PF = PF;
                r.chunks = ch;
                bool dup = false;
                for (const RowCfg& q : cands)
                    dup |= (q.TJ == r.TJ && q.PF == r.PF && q.chunks == r.chunks && q.tma == r.tma);
                if (!dup) cands.push_back(r);
            }
        }
    }
    if (N >= 128) {
        // bulk-copy (TMA) staging of the planes
        auto add_tma = [&](int TJ, int PF, int ch) {
            if (row_ctas_per_sm(N, TJ, PF) < 1) return;
            RowCfg r;
            r.TJ = TJ;
            r.PF = PF;
            r.chunks = ch;
            r.tma = 1;
            cands.push_back(r);
        };
        const int per8 = row_ctas_per_sm(N, 8, 2);
        int ch8 = (c->sms * (per8 > 0 ? per8 : 1)) / (N / 8);
        ch8 = ch8 < 1 ? 1 : (ch8 > N / 8 ? N / 8 : ch8);
        add_tma(8, 2, ch8);
        if (N <= 256) {
            int ch16 = c->sms / (N / 16);
            ch16 = ch16 < 1 ? 1 : (ch16 > N / 8 ? N / 8 : ch16);
            for (int PF : {1, 2, 3}) {
                add_tma(16, PF, ch16);
                add_tma(16, PF, 0);
            }
        }
    }
    if (c->comp) {
        std::vector<RowCfg> keep;
        for (const RowCfg& r : cands)
            if (comp_shape_ok(N, r.TJ, r.PF, r.tma)) keep.push_back(r);
        cands.swap(keep);
        if (cands.empty()) cands.push_back(default_row_cfg(c));
    }
    // save the live state into the idle FP64 buffer (the residuals of the
    // compensated form into the deltaN buffer)
    float* save = reinterpret_cast<float*>(c->f[c->cur ^ 1]);
    unsigned short* save_r = reinterpret_cast<unsigned short*>(c->dn);
    const int cur0 = c->cur;
    const SplitCtl ctl0 = *c->sctl_h;
    if (check_cuda(c, cudaMemcpyAsync(save, c->sp[cur0], sizeof(float) * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune save") ||
        check_cuda(c, cudaMemcpyAsync(save + c->gs, c->spi[cur0], sizeof(float) * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune save"))
        return IEGPU_ECUDA;
    if (c->comp &&
        (check_cuda(c, cudaMemcpyAsync(save_r, c->sxl[cur0], 2 * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune save") ||
         check_cuda(c, cudaMemcpyAsync(save_r + c->gs, c->spl[cur0], 2 * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune save")))
        return IEGPU_ECUDA;
    double best = 1e300;
    RowCfg pick = default_row_cfg(c);
    for (const RowCfg& r : cands) {
        c->row_cfg = r;
        iegpu_bg b = *bg0;
        double ms[2] = {0.0, 0.0};
        // each candidate is timed the way iegpu_leapfrog will run it: in one
        // persistent launch where its shape allows, else one launch per step
        int rc = split_profile_persist(c, 8, &b, &ms[1]);
        if (rc == 0) ms[1] *= 0.5;   // per 4 steps, as the one-step timing below
        else if (rc == 1) rc = split_profile(c, 1e300, 4, &b, ms, 2);
        // restore
        c->cur = cur0;
        *c->sctl_h = ctl0;
        if (check_cuda(c, cudaMemcpyAsync(c->sp[cur0], save, sizeof(float) * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune restore") ||
            check_cuda(c, cudaMemcpyAsync(c->spi[cur0], save + c->gs, sizeof(float) * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune restore"))
            return IEGPU_ECUDA;
        if (c->comp &&
            (check_cuda(c, cudaMemcpyAsync(c->sxl[cur0], save_r, 2 * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune restore") ||
             check_cuda(c, cudaMemcpyAsync(c->spl[cur0], save_r + c->gs, 2 * c->gs, cudaMemcpyDeviceToDevice, c->stream), "tune restore")))
            return IEGPU_ECUDA;
        if (rc) return rc;
        if (ms[1] < best) { best = ms[1]; pick = r; }
    }
    c->row_cfg = pick;
    if (sctl_up(c)) return IEGPU_ECUDA;
    split_destroy_graphs(c);
    return sync_and_check(c, "autotune");
}

int split_set_shape(iegpu_ctx* c, int rows, int prefetch, int chunks) {
    const int N = c->N;
    if (prefetch >= 10) {
        if (c->comp) return set_error(c, IEGPU_EINVAL, "the compensated form stages its planes with cp.async only");
        // bulk-copy (TMA) staging: prefetch - 10 planes ahead
        const int pf = prefetch - 10;
        const bool ok = N >= 128 && ((rows == 8 && pf == 2) || (rows == 16 && N <= 256 && pf >= 1 && pf <= 3)) &&
                        (chunks == 0 || (chunks >= 1 && chunks <= N / 8));
        if (!ok) return set_error(c, IEGPU_EINVAL, "bulk-copy shapes: rows 8 with 2 planes ahead, or rows 16 (N <= 256) with 1..3");
        const long long ctas = chunks == 0 ? balanced_ctas(c, N, rows, pf) : (long long)(N / rows) * chunks;
        if (3LL * ctas > c->part_cap || row_ctas_per_sm(N, rows, pf) < 1)
            return set_error(c, IEGPU_EINVAL, "shape does not fit this lattice's scratch");
        c->row_cfg.TJ = rows;
        c->row_cfg.PF = pf;
        c->row_cfg.chunks = chunks;
        c->row_cfg.tma = 1;
        c->tuned = 1;
        split_destroy_graphs(c);
        return IEGPU_OK;
    }
    if (N < 32 || N > 512) return set_error(c, IEGPU_EUNSUPPORTED, "the row kernel covers 32 <= N <= 512");
    if (c->comp && !comp_shape_ok(N, rows, prefetch, 0))
        return set_error(c, IEGPU_EINVAL, "compensated shapes: rows 16 (N <= 256) with prefetch 2|3, rows 8 with 2, "
                                          "rows 4 (N = 512) with 2");
    const bool plane = plane_shape(N, rows);
    const bool deep = (rows == 4 && N >= 128 && (prefetch == 3 || prefetch == 4)) ||
                      (rows == 16 && N >= 128 && N <= 256 && prefetch == 3);
    const bool balanced = chunks == 0 && !plane && N >= 128;
    const bool wide = rows == 16 && N >= 128 && N <= 256;
    if ((!plane && ((rows != 4 && rows != 8 && !wide) || ((prefetch != 1 && prefetch != 2) && !deep))) ||
        (plane && prefetch != 2 && prefetch != 4) || (!balanced && (chunks < 1 || chunks > N / 8)))
        return set_error(c, IEGPU_EINVAL,
                         "shape: rows 4|8 with prefetch 1|2 (rows 4 and N >= 128 also 3|4), rows 16 "
                         "(128 <= N <= 256) with prefetch 1..3, or rows N (N <= 64, whole planes) with "
                         "prefetch 2|4; 1 <= chunks <= N/8, or chunks 0 (N >= 128: one wave of CTAs with "
                         "equal shares)");
    const long long ctas = balanced ? balanced_ctas(c, N, rows, prefetch) : (long long)(N / rows) * chunks;
    if (3LL * ctas > c->part_cap || row_ctas_per_sm(N, rows, prefetch) < 1)
        return set_error(c, IEGPU_EINVAL, "shape does not fit this lattice's scratch");
    c->row_cfg.TJ = rows;
    c->row_cfg.PF = prefetch;
    c->row_cfg.chunks = chunks;
    c->row_cfg.tma = 0;
    c->tuned = 1;
    split_destroy_graphs(c);
    return IEGPU_OK;
}

// The host mirror of the split control holds phibar/pibar between calls; it
// is refreshed from the device after every call that changes them.
int split_leapfrog(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps, double* a_trace) {
    if (!c->tuned && max_steps > 0) {
        int rc = split_autotune(c, bg);
        if (rc) return rc;
    }
    if (steps) *steps = 0;
    if (max_steps <= 0) return max_steps < 0 ? set_error(c, IEGPU_EINVAL, "max_steps must be >= 0") : IEGPU_OK;
    if (max_steps > c->a_trace_cap) {
        if (c->a_trace) cudaFree(c->a_trace);
        c->a_trace = nullptr;
        c->a_trace_cap = 0;
        const int cap = max_steps < 1024 ? 1024 : max_steps;
        if (check_cuda(c, cudaMalloc(&c->a_trace, sizeof(double) * (size_t)cap), "a_trace alloc")) return IEGPU_ENOMEM;
        c->a_trace_cap = cap;
        split_destroy_graphs(c);
        fp64_destroy_graphs(c);
    }
    const bool persist = launch_persist(c, c->cur, 0, true) == 0;
    if (!persist && !c->sp_exec[0]) {
        int rc = split_build_graphs(c);
        if (rc) return rc;
    }
    sctl_fill(c, bg, kModeLeapfrog);
    c->sctl_h->af = af;
    c->sctl_h->steps_limit = max_steps;
    if (sctl_up(c)) return IEGPU_ECUDA;
    const int start = c->cur;
    launch_prime(c, start);  // sums of the current state -> coefficients of step 0
    if (persist) {
        for (int done = 0; done < max_steps; done += kPersistSteps) {
            const int n = max_steps - done < kPersistSteps ? max_steps - done : kPersistSteps;
            if (launch_persist(c, (start + done) & 1, n, false) != 0)
                return check_cuda(c, cudaGetLastError(), "persistent launch") ? IEGPU_ECUDA
                                                                                : set_error(c, IEGPU_ECUDA, "persistent launch");
        }
    } else {
        const int L = c->sp_steps;
        const int launches = (max_steps + L - 1) / L;
        for (int q = 0; q < launches; ++q) {
            if (check_cuda(c, cudaGraphLaunch(c->sp_exec[start], c->stream), "graph launch")) return IEGPU_ECUDA;
            c->launches += (long long)L * (c->cfg.sigw ? 2 : 1);
        }
    }
    int rc = sctl_down(c);
    const int taken = c->sctl_h->steps_done;
    c->cur = (start + taken) & 1;
    if (rc) return rc;
    sctl_bg(c, bg);
    if (steps) *steps = taken;
    if (a_trace && taken > 0 &&
        check_cuda(c, cudaMemcpy(a_trace, c->a_trace, sizeof(double) * taken, cudaMemcpyDeviceToHost), "a_trace"))
        return IEGPU_ECUDA;
    return IEGPU_OK;
}

// As split_leapfrog, launching each step kernel on its own between two CUDA
// events: ms[0] = the priming reduction, ms[1] = the step kernels' total.
int split_profile(iegpu_ctx* c, double af, int nsteps, iegpu_bg* bg, double* ms, int nk) {
    for (int q = 0; q < nk; ++q) ms[q] = 0.0;
    if (nsteps > c->a_trace_cap) {
        if (c->a_trace) cudaFree(c->a_trace);
        c->a_trace = nullptr;
        c->a_trace_cap = 0;
        const int cap = nsteps < 1024 ? 1024 : nsteps;
        if (check_cuda(c, cudaMalloc(&c->a_trace, sizeof(double) * (size_t)cap), "a_trace alloc")) return IEGPU_ENOMEM;
        c->a_trace_cap = cap;
        split_destroy_graphs(c);
        fp64_destroy_graphs(c);
    }
    sctl_fill(c, bg, kModeLeapfrog);
    c->sctl_h->af = af;
    c->sctl_h->steps_limit = nsteps;
    if (sctl_up(c)) return IEGPU_ECUDA;
    const int start = c->cur;
    float t = 0.f;
    cudaEventRecord(c->ev[1], c->stream);
    launch_prime(c, start);
    cudaEventRecord(c->ev[2], c->stream);
    if (check_cuda(c, cudaEventSynchronize(c->ev[2]), "profile")) return IEGPU_ECUDA;
    cudaEventElapsedTime(&t, c->ev[1], c->ev[2]);
    if (nk > 0) ms[0] += t;
    for (int s = 0; s < nsteps; ++s) {
        cudaEventRecord(c->ev[1], c->stream);
        launch_step(c, (start + s) & 1);
        cudaEventRecord(c->ev[2], c->stream);
        if (check_cuda(c, cudaEventSynchronize(c->ev[2]), "profile")) return IEGPU_ECUDA;
        cudaEventElapsedTime(&t, c->ev[1], c->ev[2]);
        if (nk > 1) ms[1] += t;
    }
    int rc = sctl_down(c);
    c->cur = (start + c->sctl_h->steps_done) & 1;
    if (rc) return rc;
    sctl_bg(c, bg);
    return IEGPU_OK;
}

// As split_leapfrog with persistent launches, `nsteps` steps timed between two
// CUDA events (the priming reduction before them is not timed); 1 if the
// current shape does not run persistently.
static int split_profile_persist(iegpu_ctx* c, int nsteps, iegpu_bg* bg, double* ms) {
    if (launch_persist(c, c->cur, 0, true) != 0) return 1;
    sctl_fill(c, bg, kModeLeapfrog);
    c->sctl_h->af = 1e300;
    c->sctl_h->steps_limit = nsteps;
    if (sctl_up(c)) return IEGPU_ECUDA;
    const int start = c->cur;
    launch_prime(c, start);
    cudaEventRecord(c->ev[1], c->stream);
    if (launch_persist(c, start, nsteps, false) != 0)
        return check_cuda(c, cudaGetLastError(), "persistent launch") ? IEGPU_ECUDA : set_error(c, IEGPU_ECUDA, "persistent launch");
    cudaEventRecord(c->ev[2], c->stream);
    if (check_cuda(c, cudaEventSynchronize(c->ev[2]), "profile")) return IEGPU_ECUDA;
    float t = 0.f;
    cudaEventElapsedTime(&t, c->ev[1], c->ev[2]);
    *ms = t;
    int rc = sctl_down(c);
    c->cur = (start + c->sctl_h->steps_done) & 1;
    if (rc) return rc;
    sctl_bg(c, bg);
    return IEGPU_OK;
}

int split_evolve_derivs(iegpu_ctx* c, double d, iegpu_bg* bg) {
    sctl_fill(c, bg, kModeKick);
    c->sctl_h->d_given = d;
    c->sctl_h->steps_limit = 1;
    if (sctl_up(c)) return IEGPU_ECUDA;
    launch_prime(c, c->cur);
    const unsigned grid = (unsigned)(c->gs / kThreads);
    if (c->cfg.sigw) {
        const float hodx = (float)(0.5 / (c->cfg.L / (double)c->N));
        k_split_h<<<grid, kThreads, 0, c->stream>>>(c->sp[c->cur], sigw_split(c, c->cur), c->sctl, c->lg, hodx, 1);
        c->launches++;
    }
    if (c->pot.table) k_split_kick<true><<<grid, kThreads, 0, c->stream>>>(c->sp[c->cur], c->spi[c->cur], c->sctl, c->pot, c->lg);
    else k_split_kick<false><<<grid, kThreads, 0, c->stream>>>(c->sp[c->cur], c->spi[c->cur], c->sctl, c->pot, c->lg);
    c->launches++;
    int rc = sctl_down(c);
    if (rc) return rc;
    sctl_bg(c, bg);
    return IEGPU_OK;
}

int split_evolve_fields(iegpu_ctx* c, double d, iegpu_bg* bg) {
    bg->t += d;
    SigwSplit S{};
    if (c->cfg.sigw)
        for (int q = 0; q < 6; ++q) { S.hdst[q] = c->h[c->cur][q]; S.hd[q] = c->hd[q]; }
    k_split_drift<<<(unsigned)((c->gs + 255) / 256), 256, 0, c->stream>>>(c->sp[c->cur], c->spi[c->cur], S, c->cfg.sigw,
                                                                          (long long)c->gs, d, c->sctl);
    c->launches++;
    bg->a += d * bg->ad;
    if (check_cuda(c, cudaMemcpyAsync(c->sctl_h, c->sctl, sizeof(SplitCtl), cudaMemcpyDeviceToHost, c->stream), "split ctl"))
        return IEGPU_ECUDA;
    return sync_and_check(c, "split evolve_fields");
}

// sums of the split state: [sum dphi, sum dphi^2, sum dpi, sum dpi^2, sum sq diffs, sum dV]
int split_sums(iegpu_ctx* c, double out[6]) {
    const int g = c->red_grid;
    if (c->pot.table) k_split_sums<true><<<g, kThreads, 0, c->stream>>>(c->sp[c->cur], c->spi[c->cur], c->sctl, c->pot, c->part, c->lg);
    else k_split_sums<false><<<g, kThreads, 0, c->stream>>>(c->sp[c->cur], c->spi[c->cur], c->sctl, c->pot, c->part, c->lg);
    c->launches++;
    std::vector<double> h((size_t)g * 6);
    if (check_cuda(c, cudaMemcpyAsync(h.data(), c->part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream), "split sums"))
        return IEGPU_ECUDA;
    if (check_cuda(c, cudaMemcpyAsync(c->sctl_h, c->sctl, sizeof(SplitCtl), cudaMemcpyDeviceToHost, c->stream), "split ctl"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "split sums")) return IEGPU_ECUDA;
    for (int q = 0; q < 6; ++q) out[q] = 0.0;
    for (int b = 0; b < g; ++b)
        for (int q = 0; q < 6; ++q) out[q] += h[6 * (size_t)b + q];
    return IEGPU_OK;
}

static const unsigned short* split_residual(const iegpu_ctx* c, int which) {
    if (!c->comp) return nullptr;
    return which ? c->spl[c->cur] : c->sxl[c->cur];
}

int split_materialize(iegpu_ctx* c, int which, double* out) {
    const float* x = which ? c->spi[c->cur] : c->sp[c->cur];
    k_split_materialize<<<(unsigned)((c->gs + 255) / 256), 256, 0, c->stream>>>(x, split_residual(c, which), out,
                                                                               (long long)c->gs, c->sctl, which);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "materialize");
}

int split_to_double(iegpu_ctx* c, int which, double* out) {
    const float* x = which ? c->spi[c->cur] : c->sp[c->cur];
    k_split_to_double<<<(unsigned)((c->gs + 255) / 256), 256, 0, c->stream>>>(x, split_residual(c, which), out,
                                                                             (long long)c->gs);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "to double");
}

// Takes an FP64 field already on the device: bar = its mean, x = in - bar.
int split_absorb(iegpu_ctx* c, int which, const double* in, double mean) {
    float* x = which ? c->spi[c->cur] : c->sp[c->cur];
    k_split_absorb<<<(unsigned)((c->gs + 255) / 256), 256, 0, c->stream>>>(in, x, (long long)c->gs, mean);
    c->launches++;
    if (c->comp) {
        unsigned short* r = which ? c->spl[c->cur] : c->sxl[c->cur];
        if (check_cuda(c, cudaMemsetAsync(r, 0, sizeof(unsigned short) * c->gs, c->stream), "absorb")) return IEGPU_ECUDA;
    }
    if (which) c->sctl_h->pibar = mean;
    else c->sctl_h->phibar = mean;
    // only the background fields of the control block change here
    const size_t off = which ? offsetof(SplitCtl, pibar) : offsetof(SplitCtl, phibar);
    return check_cuda(c, cudaMemcpyAsync(reinterpret_cast<char*>(c->sctl) + off, reinterpret_cast<char*>(c->sctl_h) + off,
                                         sizeof(double), cudaMemcpyHostToDevice, c->stream), "absorb");
}

}  // namespace iegpu
