// split_rows4.cuh -- the split form's vector row kernel (N = 128, 256, 512):
// its one-step and persistent kernels and their launchers, instantiated per
// lattice size in split_rows4_<N>.cu so that the shapes of the three sizes
// compile in parallel.  split_fp32.cu drives them through
// rows4_launch_<N> and rows4_persist_<N>.
#pragma once

#include "split_kernels.cuh"

namespace iegpu {

inline SplitConst split_const(const iegpu_ctx* c) {
    return make_split_const(c->cfg.dt, c->cfg.rescale_s, c->cfg.L / (double)c->N, (double)c->gs, c->pot.B2);
}

// Step buffers reading parity src and writing src ^ 1 (with the residuals in
// the compensated form).
inline SplitBufs split_bufs(const iegpu_ctx* c, int src) {
    SplitBufs B{c->sp[src], c->sp[src ^ 1], c->spi[src], c->spi[src ^ 1]};
    if (c->comp) {
        B.xls = c->sxl[src];
        B.xld = c->sxl[src ^ 1];
        B.pls = c->spl[src];
        B.pld = c->spl[src ^ 1];
    }
    return B;
}

struct StepGeom {
    int TK, TJ, CH, tiles, chunks, PF = 0, tma = 0;
    int rev = 0;   // the vector row kernel marches backwards (odd buffer parity)
    size_t smem;
    bool rows;   // full-row kernel (32 <= N <= 512)
};

template <bool TABLE, int C4, int TJ, int PF, bool TMA = false, bool COMP = false>
__global__ void __launch_bounds__((TJ + 2) * 32) k_split_rows4(SplitBufs B, SplitCtl* ctl, PotDev P, SplitConst K,
                                                               double* part, unsigned* counter, double* a_trace,
                                                               int chunks, int rev) {
    constexpr int N = 128 * C4;
    pdl_begin();
    long long u0, u1;
    if (chunks == 0) {
        // balanced: CTA c takes an equal share of the (row tile, plane) units
        const long long total = (long long)(N / TJ) * N;
        u0 = total * blockIdx.x / gridDim.x;
        u1 = total * (blockIdx.x + 1) / gridDim.x;
    } else {
        const int i0 = (int)(((long long)blockIdx.y * N) / chunks);
        const int CH = (int)(((long long)(blockIdx.y + 1) * N) / chunks) - i0;
        u0 = (long long)blockIdx.x * N + i0;
        u1 = u0 + CH;
    }
    rows4_body<TABLE, C4, TJ, PF, TMA, COMP>(B, ctl, P, K, part, counter, a_trace, u0, u1,
                                       blockIdx.x + gridDim.x * blockIdx.y, gridDim.x * gridDim.y, nullptr, rev != 0);
}

// Polls *p (acquire) until it reaches v: at most wait_limit(ctl) polls (by
// default 2^20) with a short sleep between them (about half a second in all),
// far beyond any step's length.  On giving up it marks the step
// IEGPU_ETIMEOUT, ends the call's stepping (active = 0) and returns false.
// The control block's spin_bias (a test hook, 0 otherwise) raises the target.
__device__ __forceinline__ bool spin_until(const unsigned* p, unsigned v, SplitCtl* ctl) {
    const unsigned lim = wait_limit(ctl);
    const unsigned target = v + __ldcg(&ctl->spin_bias);
    for (unsigned t = 0; t < lim; ++t) {
        if (ld_acquire(p) >= target) return true;
        __nanosleep(64);
    }
    if (atomicCAS(&ctl->error, 0, IEGPU_ETIMEOUT) == 0) ctl->errval = 0.0;
    return false;
}

// The vector row kernel for `nsteps` consecutive steps in one cooperative
// launch (every CTA resident), cp.async staging.  Step s reads the buffers of
// parity (start + s) & 1 and marches in that direction, as the one-step
// kernel.  Between steps a CTA waits until all CTAs have arrived at the step
// before (its fields are complete), issues the first copies of its range,
// and only then waits for the step's scalar update (sync[1] = s): the copies
// overlap the last CTA's sums and update.  sync[0] counts the arrivals of the
// launch; both words are zero at the launch.  The waits are made by lane 0
// of the precompute warp; a wait that gives up ends every CTA's loop.
template <bool TABLE, int C4, int TJ, int PF, bool COMP = false>
__global__ void __launch_bounds__((TJ + 2) * 32) k_split_rows4_persist(SplitBufs B0, SplitBufs B1, SplitCtl* ctl,
                                                                       PotDev P, SplitConst K, double* part,
                                                                       unsigned* sync, double* a_trace, int chunks,
                                                                       int start, int nsteps) {
    constexpr int N = 128 * C4, NTH = (TJ + 1) * 32, PHS = 3 + PF, RP = (TJ + 3) * N;
    extern __shared__ __align__(16) float smem[];
    float* ring = smem;
    float* pis = ring + PHS * RP;
    __shared__ int go_fields, go_update;
    long long u0, u1;
    if (chunks == 0) {
        const long long total = (long long)(N / TJ) * N;
        u0 = total * blockIdx.x / gridDim.x;
        u1 = total * (blockIdx.x + 1) / gridDim.x;
    } else {
        const int i0 = (int)(((long long)blockIdx.y * N) / chunks);
        const int CH = (int)(((long long)(blockIdx.y + 1) * N) / chunks) - i0;
        u0 = (long long)blockIdx.x * N + i0;
        u1 = u0 + CH;
    }
    const int slot = blockIdx.x + gridDim.x * blockIdx.y, nslots = gridDim.x * gridDim.y;
    for (int s = 0; s < nsteps; ++s) {
        const int src = (start + s) & 1;
        SplitBufs B = src ? B1 : B0;
        const bool rev = src != 0;
        if (s > 0) {
            if (threadIdx.x == NTH) go_fields = spin_until(sync, (unsigned)(s * nslots), ctl);
            __syncthreads();
            if (!go_fields) break;
            if (threadIdx.x < NTH && u0 < u1) {
                long long u = rev ? u1 : u0;
                row4_issue_start<C4, TJ, PF>(ring, pis, B, row4_march<N, TJ>(u, u0, u1, rev));
            }
            if (threadIdx.x == NTH) go_update = spin_until(sync + 1, (unsigned)s, ctl);
            __syncthreads();
            if (!go_update) {
                cp_wait<0>();
                break;
            }
        }
        StepSeq sq;
        sq.seq = sync + 1;
        sq.base = (unsigned)(s * nslots);
        sq.val = (unsigned)(s + 1);
        if (!rows4_body<TABLE, C4, TJ, PF, false, COMP>(B, ctl, P, K, part, sync, a_trace, u0, u1, slot, nslots, nullptr, rev,
                                                  s > 0, sq))
            break;
    }
}

// ---- launchers ----------------------------------------------------------

template <bool TAB, int C4, int TJV, int PFV, bool TMA = false, bool COMP = false>
static void rows4_one(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    if (smem_optin((const void*)k_split_rows4<TAB, C4, TJV, PFV, TMA, COMP>, g.smem) != cudaSuccess) {
        set_error(c, IEGPU_ECUDA, "shared memory opt-in of the split step kernel failed");   // the launch then fails
    }
    launch_pdl(k_split_rows4<TAB, C4, TJV, PFV, TMA, COMP>, grid, dim3(row4_threads(TJV)), g.smem, c->stream, B, c->sctl, c->pot,
               K, c->part, c->counter, c->a_trace, g.chunks, g.rev);
}

template <bool TAB, int C4>
static void rows4_tj(iegpu_ctx* c, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    if (c->comp) {
        // the compensated shapes (comp_shape_ok)
        if (g.TJ == 16 && C4 <= 2) {
            constexpr int CW = C4 <= 2 ? C4 : 2;
            if (g.PF == 2) rows4_one<TAB, CW, 16, 2, false, true>(c, B, K, grid, g);
            else rows4_one<TAB, CW, 16, 3, false, true>(c, B, K, grid, g);
        } else if (g.TJ == 8) {
            rows4_one<TAB, C4, 8, 2, false, true>(c, B, K, grid, g);
        } else if (C4 == 4) {
            rows4_one<TAB, 4, 4, 2, false, true>(c, B, K, grid, g);
        }
        return;
    }
    if (g.tma) {
        // bulk-copy staging: 8-row tiles with 2 planes ahead, 16-row tiles with 1..3
        if (g.TJ == 8) rows4_one<TAB, C4, 8, 2, true>(c, B, K, grid, g);
        else if (C4 <= 2) {
            constexpr int CW = C4 <= 2 ? C4 : 2;
            if (g.PF == 1) rows4_one<TAB, CW, 16, 1, true>(c, B, K, grid, g);
            else if (g.PF == 2) rows4_one<TAB, CW, 16, 2, true>(c, B, K, grid, g);
            else rows4_one<TAB, CW, 16, 3, true>(c, B, K, grid, g);
        }
        return;
    }
    if (g.TJ == 4) {
        switch (g.PF) {
            case 1: rows4_one<TAB, C4, 4, 1>(c, B, K, grid, g); break;
            case 2: rows4_one<TAB, C4, 4, 2>(c, B, K, grid, g); break;
            case 3: rows4_one<TAB, C4, 4, 3>(c, B, K, grid, g); break;
            default: rows4_one<TAB, C4, 4, 4>(c, B, K, grid, g); break;
        }
    } else if (g.TJ == 8) {
        if (g.PF == 1) rows4_one<TAB, C4, 8, 1>(c, B, K, grid, g); else rows4_one<TAB, C4, 8, 2>(c, B, K, grid, g);
    } else if (C4 <= 2) {
        // 16-row tiles: one CTA of 18 warps per SM
        if (g.PF == 1) rows4_one<TAB, (C4 <= 2 ? C4 : 2), 16, 1>(c, B, K, grid, g);
        else if (g.PF == 2) rows4_one<TAB, (C4 <= 2 ? C4 : 2), 16, 2>(c, B, K, grid, g);
        else rows4_one<TAB, (C4 <= 2 ? C4 : 2), 16, 3>(c, B, K, grid, g);
    }
}

constexpr int kPersistSteps = 64;   // steps per cooperative launch

// Launches k_split_rows4_persist of one shape for `nsteps` steps from buffer
// parity `start`; 1 if the shape's grid is not resident all at once (the
// caller then steps kernel by kernel), -1 on a launch error.
template <bool TAB, int C4, int TJV, int PFV, bool COMP = false>
static int persist_one(iegpu_ctx* c, int start, int nsteps, dim3 grid, const StepGeom& g, bool check_only) {
    auto kern = k_split_rows4_persist<TAB, C4, TJV, PFV, COMP>;
    if (smem_optin((const void*)kern, g.smem) != cudaSuccess)
        return set_error(c, IEGPU_ECUDA, "shared memory opt-in of the split step kernel failed");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, row4_threads(TJV), g.smem) != cudaSuccess ||
        (long long)per_sm * c->sms < (long long)grid.x * grid.y) {
        cudaGetLastError();
        return 1;
    }
    if (check_only) return 0;
    const SplitConst K = split_const(c);
    const SplitBufs B0 = split_bufs(c, 0);
    const SplitBufs B1 = split_bufs(c, 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(row4_threads(TJV));
    cfg.dynamicSmemBytes = g.smem;
    cfg.stream = c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    unsigned* sync = c->counter + 2;
    if (cudaMemsetAsync(sync, 0, 2 * sizeof(unsigned), c->stream) != cudaSuccess) return -1;
    if (cudaLaunchKernelEx(&cfg, kern, B0, B1, c->sctl, c->pot, K, c->part, sync, c->a_trace, g.chunks, start,
                           nsteps) != cudaSuccess)
        return -1;
    c->launches++;
    return 0;
}

template <bool TAB, int C4>
static int persist_tj(iegpu_ctx* c, int start, int nsteps, dim3 grid, const StepGeom& g, bool check_only) {
    if (c->comp) {
        if (g.TJ == 16 && C4 <= 2) {
            constexpr int CW = C4 <= 2 ? C4 : 2;
            if (g.PF == 2) return persist_one<TAB, CW, 16, 2, true>(c, start, nsteps, grid, g, check_only);
            return persist_one<TAB, CW, 16, 3, true>(c, start, nsteps, grid, g, check_only);
        }
        if (g.TJ == 8 && C4 <= 2) return persist_one<TAB, C4, 8, 2, true>(c, start, nsteps, grid, g, check_only);
        return 1;
    }
    if (g.TJ == 4) {
        switch (g.PF) {
            case 1: return persist_one<TAB, C4, 4, 1>(c, start, nsteps, grid, g, check_only);
            case 2: return persist_one<TAB, C4, 4, 2>(c, start, nsteps, grid, g, check_only);
            case 3: return persist_one<TAB, C4, 4, 3>(c, start, nsteps, grid, g, check_only);
            default: return persist_one<TAB, C4, 4, 4>(c, start, nsteps, grid, g, check_only);
        }
    }
    if (g.TJ == 8) {
        if (g.PF == 1) return persist_one<TAB, C4, 8, 1>(c, start, nsteps, grid, g, check_only);
        return persist_one<TAB, C4, 8, 2>(c, start, nsteps, grid, g, check_only);
    }
    if (C4 <= 2) {
        constexpr int CW = C4 <= 2 ? C4 : 2;
        if (g.PF == 1) return persist_one<TAB, CW, 16, 1>(c, start, nsteps, grid, g, check_only);
        if (g.PF == 2) return persist_one<TAB, CW, 16, 2>(c, start, nsteps, grid, g, check_only);
        return persist_one<TAB, CW, 16, 3>(c, start, nsteps, grid, g, check_only);
    }
    return 1;
}

// One step of the vector row kernel of the current shape (tab: tabulated
// potential), and up to nsteps steps in one cooperative launch (0: launched,
// or would launch with check_only; 1: the shape's grid is not resident at
// once; -1 or an error code: launch error).
void rows4_launch_128(iegpu_ctx* c, bool tab, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g);
void rows4_launch_256(iegpu_ctx* c, bool tab, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g);
void rows4_launch_512(iegpu_ctx* c, bool tab, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g);
int rows4_persist_128(iegpu_ctx* c, bool tab, int start, int nsteps, dim3 grid, const StepGeom& g, bool check_only);
int rows4_persist_256(iegpu_ctx* c, bool tab, int start, int nsteps, dim3 grid, const StepGeom& g, bool check_only);
int rows4_persist_512(iegpu_ctx* c, bool tab, int start, int nsteps, dim3 grid, const StepGeom& g, bool check_only);

}  // namespace iegpu
