// ensemble.cu -- many independent lattices (seeds, lattice sizes) evolved
// together in the split form.
//
// The reference runs one lattice per process.  Here an ensemble of lattices
// of N = 32 .. 256 lives in one set of concatenated device arrays and one
// kernel launch advances every lattice by one leapfrog step: each CTA looks
// up its (lattice, tile) pair in a work table and runs the same row-tile step
// body as the one-lattice split form, so a lattice of the ensemble gives the
// same bits as a one-lattice run with the same tile shape.  Every lattice
// keeps its own background (a, ad, t, phibar, pibar), its own stop condition
// (a > af of that lattice, or the step limit) and its own reduction: the last
// CTA of a lattice to finish a step adds that lattice's partial sums and runs
// its Friedmann update.  Lattices that have stopped drop out of the work
// table between CUDA-graph launches (a graph holds L steps).  The launch
// shape -- rows per tile, planes prefetched and plane chunks per lattice --
// is chosen by an autotuner that times candidate shapes on the live state.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ensemble.cuh"
#include "split_kernels.cuh"

namespace iegpu {

struct EnsArgs {
    float* x[2];
    float* p[2];
    SplitCtl* ctl;
    int* cur;
    const EnsLat* lat;
    double* part;
    unsigned* counter;
    PotDev P;
};

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Sums of each lattice's current dphi and the coefficients of its first step.
template <bool TABLE>
__global__ void __launch_bounds__(kThreads) k_ens_prime(EnsArgs A, const int2* __restrict__ pwork) {
    const int2 w = pwork[blockIdx.x];
    const EnsLat& L = A.lat[w.x];
    const float* x = A.x[A.cur[w.x] & 1] + L.off;
    prime_body<TABLE>(x, A.ctl + w.x, A.P, L.K, A.part + 3LL * L.part_off, A.counter + w.x, nullptr, L.lg, w.y,
                      L.pslots, A.cur + w.x);
}

// One leapfrog step of every lattice in a class's work table: the CTA's
// (lattice, tile) pair, its buffers and plane range.
struct EnsTile {
    SplitBufs B;
    SplitCtl* ctl;
    double* part;
    unsigned* cnt;
    int* st;
    SplitConst K;
    int j0, i0, CH, slot, nslots;
};

__device__ __forceinline__ EnsTile ens_tile(const EnsArgs& A, const int2* work, int TJ) {
    const int2 w = work[blockIdx.x];
    const EnsLat& L = A.lat[w.x];
    const int c = A.cur[w.x] & 1;
    EnsTile t;
    t.B = SplitBufs{A.x[c] + L.off, A.x[c ^ 1] + L.off, A.p[c] + L.off, A.p[c ^ 1] + L.off};
    const int N = 1 << L.lg;
    const int rt = w.y % L.rowtiles, ch = w.y / L.rowtiles;
    t.j0 = rt * TJ;
    t.i0 = (int)(((long long)ch * N) / L.chunks);
    t.CH = (int)(((long long)(ch + 1) * N) / L.chunks) - t.i0;
    t.ctl = A.ctl + w.x;
    t.part = A.part + 3LL * L.part_off;
    t.cnt = A.counter + w.x;
    t.st = A.cur + w.x;
    t.K = L.K;
    t.slot = w.y;
    t.nslots = L.tiles;
    return t;
}

template <bool TABLE, int C, int TJ, int PF>
__global__ void __launch_bounds__((TJ + 1) * 32) k_ens_rows(EnsArgs A, const int2* __restrict__ work) {
    pdl_begin();
    const EnsTile t = ens_tile(A, work, TJ);
    rows_body<TABLE, C, TJ, PF>(t.B, t.ctl, A.P, t.K, t.part, t.cnt, nullptr, t.j0, t.i0, t.CH, t.slot, t.nslots, t.st);
}

template <bool TABLE, int C4, int TJ, int PF>
__global__ void __launch_bounds__((TJ + 2) * 32) k_ens_rows4(EnsArgs A, const int2* __restrict__ work) {
    pdl_begin();
    const EnsTile t = ens_tile(A, work, TJ);
    constexpr int N = 128 * C4;
    const long long u0 = (long long)(t.j0 / TJ) * N + t.i0;
    // the march direction follows the lattice's buffer parity, as in the one-lattice kernel
    rows4_body<TABLE, C4, TJ, PF>(t.B, t.ctl, A.P, t.K, t.part, t.cnt, nullptr, u0, u0 + t.CH, t.slot, t.nslots, t.st,
                                  (*t.st & 1) != 0);
}

template <bool TABLE, int N, int NT, int PF>
__global__ void __launch_bounds__(NT, plane_min_ctas(N)) k_ens_plane(EnsArgs A, const int2* __restrict__ work) {
    pdl_begin();
    const EnsTile t = ens_tile(A, work, N);
    plane_body<TABLE, N, NT, PF>(t.B, t.ctl, A.P, t.K, t.part, t.cnt, nullptr, t.i0, t.CH, t.slot, t.nslots, t.st);
}

// Persistent ensemble step: one cooperative launch advances every lattice by
// up to `nsteps` leapfrog steps.  Item q of the launch is step q / nitems of
// entry q % nitems of `queue` (one step's (lattice, tile) pairs, the largest
// lattices first); CTAs claim items in order from qsync[0].  Before an item of
// step s a CTA waits until its lattice's update of step s - 1 is published
// (qsync[2 + b] >= s, written by the lattice's last CTA of that step after
// its Friedmann update) or the lattice has stopped.  Items are claimed in
// queue order and an item waits only for items earlier in the queue, which
// resident CTAs hold, so every wait ends; it is still bounded (`polls`), after
// which the lattice's step is marked IEGPU_ETIMEOUT, qsync[1] is raised and
// every CTA leaves.  Every lattice runs the 8-row tile body of its size and
// its scalar update with the one-lattice arithmetic.
constexpr int kEnsPersistTJ = 8, kEnsPersistPF = 2;

__device__ __forceinline__ int ld_acquire_int(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <bool TABLE>
__global__ void __launch_bounds__((kEnsPersistTJ + 1) * 32, 3) k_ens_persist(EnsArgs A, const int2* __restrict__ queue,
                                                                         int nitems, int nsteps, unsigned* qsync,
                                                                         unsigned polls) {
    constexpr int TJ = kEnsPersistTJ, PF = kEnsPersistPF;
    __shared__ int item_s, go_s;
    unsigned* done_step = qsync + 2;
    const long long total = (long long)nitems * nsteps;
    for (;;) {
        if (threadIdx.x == 0) item_s = (int)atomicAdd(qsync, 1u);
        __syncthreads();
        const long long q = item_s;
        if (q >= total) break;
        const int s = (int)(q / nitems);
        const int2 w = queue[q % nitems];
        const int b = w.x;
        if (threadIdx.x == 0) {
            int go = 0;   // 1: step the item; 2: the lattice has stopped; 0: leave
            for (unsigned t = 0; t < polls; ++t) {
                if (ld_acquire(qsync + 1)) break;
                if (ld_acquire_int(A.cur + b) & 2) { go = 2; break; }
                if (ld_acquire(done_step + b) >= (unsigned)s) { go = 1; break; }
                __nanosleep(64);
            }
            if (go == 0 && !ld_acquire(qsync + 1)) {
                if (atomicCAS(&A.ctl[b].error, 0, IEGPU_ETIMEOUT) == 0) A.ctl[b].errval = 0.0;
                atomicExch(qsync + 1, 1u);
            }
            go_s = go;
        }
        __syncthreads();
        if (go_s == 0) break;
        if (go_s == 1) {
            const EnsLat& L = A.lat[b];
            const int c = __ldcg(A.cur + b) & 1;
            const SplitBufs B{A.x[c] + L.off, A.x[c ^ 1] + L.off, A.p[c] + L.off, A.p[c ^ 1] + L.off};
            const int N = 1 << L.lg;
            const int rt = w.y % L.rowtiles, ch = w.y / L.rowtiles;
            const int i0 = (int)(((long long)ch * N) / L.chunks);
            const int CH = (int)(((long long)(ch + 1) * N) / L.chunks) - i0;
            StepSeq sq;
            sq.seq = done_step + b;
            sq.base = (unsigned)s * (unsigned)L.tiles;
            sq.val = (unsigned)(s + 1);
            SplitCtl* ctl = A.ctl + b;
            double* part = A.part + 3LL * L.part_off;
            switch (L.lg) {
                case 5: rows_body<TABLE, 1, TJ, PF>(B, ctl, A.P, L.K, part, A.counter + b, nullptr, rt * TJ, i0, CH, w.y,
                                                    L.tiles, A.cur + b, sq); break;
                case 6: rows_body<TABLE, 2, TJ, PF>(B, ctl, A.P, L.K, part, A.counter + b, nullptr, rt * TJ, i0, CH, w.y,
                                                    L.tiles, A.cur + b, sq); break;
                default: rows_body<TABLE, 4, TJ, PF>(B, ctl, A.P, L.K, part, A.counter + b, nullptr, rt * TJ, i0, CH,
                                                     w.y, L.tiles, A.cur + b, sq); break;
            }
        }
        __syncthreads();   // the item's shared memory is free before the next claim
    }
}

// evolve_fields of every lattice with its own step d[b]: dphi += d dpi and
// phibar += d pibar (the one-lattice split drift, lattice by lattice).
__global__ void __launch_bounds__(256) k_ens_drift(EnsArgs A, const double* __restrict__ d, int count) {
    __shared__ int b_s;
    const long long first = (long long)blockIdx.x * 256;
    if (threadIdx.x == 0) b_s = ens_lattice_of(A.lat, count, first);
    __syncthreads();
    const int b = b_s;
    const long long id = first + threadIdx.x;
    const double db = d[b];
    if (id == A.lat[b].off) A.ctl[b].phibar = A.ctl[b].phibar + db * A.ctl[b].pibar;
    const int c = A.cur[b] & 1;
    const float df = (float)db;
    A.x[c][id] = A.x[c][id] + df * A.p[c][id];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

int ens_error(iegpu_ens* e, int code, const char* fmt, ...) {
    char buf[600];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    e->err = buf;
    return code;
}

int ens_cuda(iegpu_ens* e, cudaError_t err, const char* what) {
    if (err == cudaSuccess) return IEGPU_OK;
    cudaGetLastError();
    return ens_error(e, err == cudaErrorMemoryAllocation ? IEGPU_ENOMEM : IEGPU_ECUDA, "%s: %s", what,
                     cudaGetErrorString(err));
}

static int ens_sync(iegpu_ens* e, const char* what) {
    if (int rc = ens_cuda(e, cudaGetLastError(), what)) return rc;
    return ens_cuda(e, cudaStreamSynchronize(e->stream), what);
}

template <typename T>
static int ens_alloc(iegpu_ens* e, T** p, size_t n) {
    return ens_cuda(e, cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (n ? n : 1)), "device alloc");
}

static iegpu_ctx* ens_helper(const iegpu_ens* e, int N) {
    for (size_t q = 0; q < e->sizes.size(); ++q)
        if (e->sizes[q] == N) return e->helper[q];
    return nullptr;
}

static EnsArgs ens_args(const iegpu_ens* e) {
    EnsArgs A;
    A.x[0] = e->x[0];
    A.x[1] = e->x[1];
    A.p[0] = e->p[0];
    A.p[1] = e->p[1];
    A.ctl = e->ctl;
    A.cur = e->cur;
    A.lat = e->lat;
    A.part = e->part;
    A.counter = e->counter;
    A.P = e->helper[0]->pot;
    return A;
}

// The one-lattice priming grid for N (sums in the same slot order).
static int ens_prime_slots(const iegpu_ens* e, int N) {
    const long long sites = (long long)N * N * N;
    int g = e->sms * 4;
    if (g * 256LL > sites) g = (int)((sites + 255) / 256);
    return g;
}

// Launch shapes, as in the one-lattice form: TJ rows per tile (4 or 8) with
// PF = 1 or 2 planes prefetched (4-row tiles at N >= 128 also 3 or 4), 16-row
// tiles at 128 <= N <= 256 with PF = 1 to 3, or TJ = N (N = 32, 64) for whole
// planes with PF = 2 or 4.
static bool ens_plane(int N, int TJ) { return TJ == N && (N == 32 || N == 64); }
static int ens_threads(int N, int TJ) {
    return ens_plane(N, TJ) ? plane_nt(N) : N >= 128 ? row4_threads(TJ) : (TJ + 1) * 32;
}

static size_t ens_smem(int N, int TJ, int PF) {
    if (ens_plane(N, TJ)) return sizeof(float) * (size_t)split_plane_smem_floats(N, PF);
    return sizeof(float) * (size_t)(N >= 128 ? split_row4_smem_floats(TJ, N, PF) : split_row_smem_floats(TJ, N, PF));
}

static bool ens_shape_ok(int N, int TJ, int PF, int chunks) {
    if (chunks < 1 || chunks > N / 8) return false;
    if (ens_plane(N, TJ)) return PF == 2 || PF == 4;
    const bool deep = TJ == 4 && N >= 128 && (PF == 3 || PF == 4);
    if (TJ == 16) return N >= 128 && N <= 256 && PF >= 1 && PF <= 3 && ens_smem(N, TJ, PF) <= 227 * 1024;
    return (TJ == 4 || TJ == 8) && (PF == 1 || PF == 2 || deep) && ens_smem(N, TJ, PF) <= 227 * 1024;
}

static void ens_destroy_graph(iegpu_ens* e) {
    if (e->exec) cudaGraphExecDestroy(e->exec);
    e->exec = nullptr;
    for (EnsClass& c : e->cls) c.graph_nwork = -1;
}

// Kernel of a class's shape, launched over its work table on `st`.
template <bool TAB>
static int ens_launch_class(iegpu_ens* e, const EnsClass& c, const EnsArgs& A, cudaStream_t st, bool set_attr) {
    const int N = c.N, TJ = c.TJ, PF = c.PF;
    const unsigned grid = (unsigned)(c.nwork > 0 ? c.nwork : 1);
    const int nthr = ens_threads(N, TJ);
    const void* fn = nullptr;
#define IEGPU_ENS_PICK(KERNEL) \
    do {                                                                                                   \
        fn = reinterpret_cast<const void*>(&KERNEL);                                                       \
        if (!set_attr) launch_pdl(KERNEL, dim3(grid), dim3(nthr), c.smem, st, A, (const int2*)c.work);     \
    } while (0)
    if (ens_plane(N, TJ)) {
        if (N == 32) { if (PF == 4) IEGPU_ENS_PICK((k_ens_plane<TAB, 32, plane_nt(32), 4>)); else IEGPU_ENS_PICK((k_ens_plane<TAB, 32, plane_nt(32), 2>)); }
        else { if (PF == 4) IEGPU_ENS_PICK((k_ens_plane<TAB, 64, plane_nt(64), 4>)); else IEGPU_ENS_PICK((k_ens_plane<TAB, 64, plane_nt(64), 2>)); }
    } else if (N == 32) {
        if (TJ == 4) { if (PF == 1) IEGPU_ENS_PICK((k_ens_rows<TAB, 1, 4, 1>)); else IEGPU_ENS_PICK((k_ens_rows<TAB, 1, 4, 2>)); }
        else { if (PF == 1) IEGPU_ENS_PICK((k_ens_rows<TAB, 1, 8, 1>)); else IEGPU_ENS_PICK((k_ens_rows<TAB, 1, 8, 2>)); }
    } else if (N == 64) {
        if (TJ == 4) { if (PF == 1) IEGPU_ENS_PICK((k_ens_rows<TAB, 2, 4, 1>)); else IEGPU_ENS_PICK((k_ens_rows<TAB, 2, 4, 2>)); }
        else { if (PF == 1) IEGPU_ENS_PICK((k_ens_rows<TAB, 2, 8, 1>)); else IEGPU_ENS_PICK((k_ens_rows<TAB, 2, 8, 2>)); }
    } else if (N == 128) {
        if (TJ == 4) {
            if (PF == 1) IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 4, 1>));
            else if (PF == 2) IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 4, 2>));
            else if (PF == 3) IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 4, 3>));
            else IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 4, 4>));
        } else if (TJ == 16) {
            if (PF == 1) IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 16, 1>));
            else if (PF == 2) IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 16, 2>));
            else IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 16, 3>));
        } else { if (PF == 1) IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 8, 1>)); else IEGPU_ENS_PICK((k_ens_rows4<TAB, 1, 8, 2>)); }
    } else {
        if (TJ == 4) {
            if (PF == 1) IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 4, 1>));
            else if (PF == 2) IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 4, 2>));
            else if (PF == 3) IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 4, 3>));
            else IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 4, 4>));
        } else if (TJ == 16) {
            if (PF == 1) IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 16, 1>));
            else if (PF == 2) IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 16, 2>));
            else IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 16, 3>));
        } else { if (PF == 1) IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 8, 1>)); else IEGPU_ENS_PICK((k_ens_rows4<TAB, 2, 8, 2>)); }
    }
#undef IEGPU_ENS_PICK
    if (set_attr)
        return ens_cuda(e, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem),
                        "shared memory attribute");
    return IEGPU_OK;
}

// Per-lattice descriptors and per-class shared memory for the current shapes.
static int ens_layout(iegpu_ens* e) {
    std::vector<int2> pw;
    long long slots = 0;
    e->lat_h.assign((size_t)e->count, EnsLat{});
    for (int b = 0; b < e->count; ++b) {
        const int N = e->N[(size_t)b];
        const EnsClass& c = e->cls[(size_t)e->cls_of[(size_t)b]];
        EnsLat& L = e->lat_h[(size_t)b];
        L.off = e->off[(size_t)b];
        L.lg = 0;
        while ((1 << L.lg) < N) ++L.lg;
        L.rowtiles = N / c.TJ;
        L.chunks = c.chunks;
        L.tiles = L.rowtiles * L.chunks;
        L.pslots = ens_prime_slots(e, N);
        L.part_off = (int)slots;
        slots += std::max(L.tiles, L.pslots);
        L.K = make_split_const(e->cfg.dt, e->cfg.rescale_s, e->cfg.L / (double)N, (double)N * N * N,
                               e->helper[0]->pot.B2);
        for (int s = 0; s < L.pslots; ++s) pw.push_back(make_int2(b, s));
    }
    if (int rc = ens_sync(e, "ensemble layout")) return rc;
    if ((size_t)(3 * slots) > e->part_cap) {
        if (e->part) cudaFree(e->part);
        e->part = nullptr;
        e->part_cap = 0;
        if (int rc = ens_alloc(e, &e->part, (size_t)(3 * slots))) return rc;
        e->part_cap = (size_t)(3 * slots);
    }
    if ((int)pw.size() > e->npwork) {
        if (e->pwork) cudaFree(e->pwork);
        e->pwork = nullptr;
        if (int rc = ens_alloc(e, &e->pwork, pw.size())) return rc;
    }
    e->npwork = (int)pw.size();
    if (int rc = ens_cuda(e, cudaMemcpyAsync(e->pwork, pw.data(), sizeof(int2) * pw.size(), cudaMemcpyHostToDevice,
                                             e->stream), "prime table"))
        return rc;
    if (int rc = ens_cuda(e, cudaMemcpyAsync(e->lat, e->lat_h.data(), sizeof(EnsLat) * (size_t)e->count,
                                             cudaMemcpyHostToDevice, e->stream), "lattice table"))
        return rc;
    ens_destroy_graph(e);
    const EnsArgs A = ens_args(e);
    for (EnsClass& c : e->cls) {
        c.smem = ens_smem(c.N, c.TJ, c.PF);
        // set outside any stream capture
        const int rc = A.P.table ? ens_launch_class<true>(e, c, A, e->stream, true)
                                 : ens_launch_class<false>(e, c, A, e->stream, true);
        if (rc) return rc;
    }
    return ens_sync(e, "ensemble layout");
}

// Work tables over the lattices with active[b] (stream-ordered copies).
static int ens_work(iegpu_ens* e, const std::vector<char>& active) {
    for (EnsClass& c : e->cls) {
        std::vector<int2> w;
        for (int b : c.lats)
            if (active[(size_t)b])
                for (int t = 0; t < e->lat_h[(size_t)b].tiles; ++t) w.push_back(make_int2(b, t));
        if ((int)w.size() > c.work_cap) {
            if (int rc = ens_sync(e, "work table")) return rc;
            if (c.work) cudaFree(c.work);
            c.work = nullptr;
            c.work_cap = 0;
            if (int rc = ens_alloc(e, &c.work, w.size())) return rc;
            c.work_cap = (int)w.size();
            ens_destroy_graph(e);
        }
        c.nwork = (int)w.size();
        if (!w.empty())
            if (int rc = ens_cuda(e, cudaMemcpyAsync(c.work, w.data(), sizeof(int2) * w.size(), cudaMemcpyHostToDevice,
                                                     e->stream), "work table"))
                return rc;
    }
    return IEGPU_OK;
}

// One step of every class: fork from the main stream, one kernel per class on
// its own stream, join back.
static int ens_launch_step(iegpu_ens* e) {
    const EnsArgs A = ens_args(e);
    if (int rc = ens_cuda(e, cudaEventRecord(e->fork, e->stream), "fork")) return rc;
    for (EnsClass& c : e->cls) {
        if (c.nwork == 0) continue;
        if (int rc = ens_cuda(e, cudaStreamWaitEvent(c.stream, e->fork, 0), "fork")) return rc;
        const int rc = A.P.table ? ens_launch_class<true>(e, c, A, c.stream, false)
                                 : ens_launch_class<false>(e, c, A, c.stream, false);
        if (rc) return rc;
        e->launches++;
        if (int r2 = ens_cuda(e, cudaEventRecord(c.done, c.stream), "join")) return r2;
        if (int r2 = ens_cuda(e, cudaStreamWaitEvent(e->stream, c.done, 0), "join")) return r2;
    }
    return IEGPU_OK;
}

static void ens_launch_prime(iegpu_ens* e) {
    const EnsArgs A = ens_args(e);
    if (A.P.table) k_ens_prime<true><<<e->npwork, kThreads, 0, e->stream>>>(A, e->pwork);
    else k_ens_prime<false><<<e->npwork, kThreads, 0, e->stream>>>(A, e->pwork);
    e->launches++;
}

static constexpr int kEnsGraphSteps = 16;

// L steps as a graph: every class is an independent chain of L kernels.
static int ens_build_graph(iegpu_ens* e) {
    ens_destroy_graph(e);
    const EnsArgs A = ens_args(e);
    cudaGraph_t g;
    if (int rc = ens_cuda(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal), "graph capture"))
        return rc;
    int rc = ens_cuda(e, cudaEventRecord(e->fork, e->stream), "fork");
    for (EnsClass& c : e->cls) {
        if (rc || c.nwork == 0) continue;
        rc = ens_cuda(e, cudaStreamWaitEvent(c.stream, e->fork, 0), "fork");
        for (int s = 0; s < kEnsGraphSteps && !rc; ++s)
            rc = A.P.table ? ens_launch_class<true>(e, c, A, c.stream, false)
                           : ens_launch_class<false>(e, c, A, c.stream, false);
        if (!rc) rc = ens_cuda(e, cudaEventRecord(c.done, c.stream), "join");
        if (!rc) rc = ens_cuda(e, cudaStreamWaitEvent(e->stream, c.done, 0), "join");
    }
    const int rc_end = ens_cuda(e, cudaStreamEndCapture(e->stream, &g), "graph capture end");
    if (rc) {
        if (!rc_end) cudaGraphDestroy(g);
        return rc;
    }
    if (rc_end) return rc_end;
    const cudaError_t err = cudaGraphInstantiate(&e->exec, g, 0);
    cudaGraphDestroy(g);
    if (int r2 = ens_cuda(e, err, "graph instantiate")) return r2;
    e->graph_steps = kEnsGraphSteps;
    for (EnsClass& c : e->cls) c.graph_nwork = c.nwork;
    return IEGPU_OK;
}

static bool ens_graph_current(const iegpu_ens* e) {
    if (!e->exec) return false;
    for (const EnsClass& c : e->cls)
        if (c.graph_nwork != c.nwork) return false;
    return true;
}

static void ens_fill(iegpu_ens* e, const iegpu_bg* bg, const double* af, int max_steps) {
    for (int b = 0; b < e->count; ++b) {
        SplitCtl& C = e->ctl_h[b];
        C.bg.t = bg[b].t;
        C.bg.a = bg[b].a;
        C.bg.ad = bg[b].ad;
        C.bg.ad2 = bg[b].ad2;
        C.bg.astep = bg[b].astep;
        C.mode = kModeLeapfrog;
        C.steps_done = 0;
        C.steps_limit = max_steps;
        C.done = 0;
        C.error = 0;
        C.active = 0;
        C.pre_claim = 0;
        C.pre.ok = 0;
        C.deferred = 0;
        C.af = af ? af[b] : 1e300;
        e->cur_h[b] &= 1;
    }
}

static int ens_upload_ctl(iegpu_ens* e) {
    if (int rc = ens_cuda(e, cudaMemcpyAsync(e->ctl, e->ctl_h, sizeof(SplitCtl) * (size_t)e->count,
                                             cudaMemcpyHostToDevice, e->stream), "control upload"))
        return rc;
    return ens_cuda(e, cudaMemcpyAsync(e->cur, e->cur_h, sizeof(int) * (size_t)e->count, cudaMemcpyHostToDevice,
                                       e->stream), "state upload");
}

static int ens_download_ctl(iegpu_ens* e) {
    if (int rc = ens_cuda(e, cudaMemcpyAsync(e->ctl_h, e->ctl, sizeof(SplitCtl) * (size_t)e->count,
                                             cudaMemcpyDeviceToHost, e->stream), "control download"))
        return rc;
    if (int rc = ens_cuda(e, cudaMemcpyAsync(e->cur_h, e->cur, sizeof(int) * (size_t)e->count, cudaMemcpyDeviceToHost,
                                             e->stream), "state download"))
        return rc;
    return ens_sync(e, "ensemble control");
}

static int ens_finish(iegpu_ens* e, iegpu_bg* bg, int* steps) {
    if (int rc = ens_download_ctl(e)) return rc;
    for (int b = 0; b < e->count; ++b) {
        const SplitCtl& C = e->ctl_h[b];
        bg[b].t = C.bg.t;
        bg[b].a = C.bg.a;
        bg[b].ad = C.bg.ad;
        bg[b].ad2 = C.bg.ad2;
        bg[b].astep = C.bg.astep;
        if (steps) steps[b] = C.steps_done;
    }
    for (int b = 0; b < e->count; ++b) {
        const SplitCtl& C = e->ctl_h[b];
        if (C.deferred)
            return ens_error(e, IEGPU_ECUDA, "internal: a scalar update of lattice %d was left unapplied", b);
        if (C.error == IEGPU_ERANGE) {
            const iegpu_ctx* h = e->helper[0];
            return ens_error(e, IEGPU_ERANGE,
                             "Field value near %.17g is outside the numerical potential range [%.17g, %.17g] (lattice %d).\n",
                             C.errval, h->htab_x.empty() ? 0.0 : h->htab_x.back(),
                             h->htab_x.empty() ? 0.0 : h->htab_x.front(), b);
        }
    }
    return IEGPU_OK;
}

// Steps the lattices of the classes in `which` (all if empty) one launch
// at a time with CUDA events around every step: ms[0] = priming reduction,
// ms[1] = the steps' total device time (classes side by side).
static int ens_profile(iegpu_ens* e, const double* af, int nsteps, iegpu_bg* bg, double ms[2], int only_class) {
    ms[0] = ms[1] = 0.0;
    ens_fill(e, bg, af, nsteps);
    if (int rc = ens_upload_ctl(e)) return rc;
    std::vector<char> act((size_t)e->count, 1);
    if (only_class >= 0)
        for (int b = 0; b < e->count; ++b) act[(size_t)b] = e->cls_of[(size_t)b] == only_class;
    if (int rc = ens_work(e, act)) return rc;
    float t = 0.f;
    cudaEventRecord(e->ev[0], e->stream);
    ens_launch_prime(e);
    cudaEventRecord(e->ev[1], e->stream);
    if (int rc = ens_cuda(e, cudaEventSynchronize(e->ev[1]), "profile")) return rc;
    cudaEventElapsedTime(&t, e->ev[0], e->ev[1]);
    ms[0] = t;
    for (int s = 0; s < nsteps; ++s) {
        cudaEventRecord(e->ev[0], e->stream);
        if (int rc = ens_launch_step(e)) return rc;
        cudaEventRecord(e->ev[1], e->stream);
        if (int rc = ens_cuda(e, cudaEventSynchronize(e->ev[1]), "profile")) return rc;
        cudaEventElapsedTime(&t, e->ev[0], e->ev[1]);
        ms[1] += t;
    }
    return ens_finish(e, bg, nullptr);
}

// Candidate shapes of a class of size N.
static std::vector<int3> ens_candidates(const iegpu_ens* e, int N, int nlat) {
    std::vector<int3> out;   // (TJ, PF, chunks)
    auto add = [&](int TJ, int PF, int ch) {
        if (ch > N / 8) ch = N / 8;
        if (ch < 1) ch = 1;
        if (!ens_shape_ok(N, TJ, PF, ch)) return;
        for (const int3& q : out)
            if (q.x == TJ && q.y == PF && q.z == ch) return;
        out.push_back(make_int3(TJ, PF, ch));
    };
    if (N <= 64)
        for (int PF : {2, 4})
            for (int ch = N / 8; ch >= 1; ch /= 2) add(N, PF, ch);
    for (int TJ : {4, 8})
        for (int PF : {1, 2, 3, 4}) {
            if (PF > 2 && (TJ != 4 || N < 128)) continue;
            // one or two waves of the whole class at an estimated 3 CTAs per SM
            const int per_lat = N / TJ;
            for (int waves : {1, 2}) add(TJ, PF, (waves * 3 * e->sms) / (per_lat * (nlat > 0 ? nlat : 1)));
        }
    // 16-row tiles are accepted by iegpu_ens_set_shape but not tuned over: for
    // the 8 x 128^3 class they measured slower than 8-row tiles (154 vs 145 us).
    return out;
}

static int ens_autotune(iegpu_ens* e, const iegpu_bg* bg0) {
    // save the live state (both halves: lattices may sit in either) into the FP64 arrays
    const size_t n = (size_t)e->total;
    float* save = reinterpret_cast<float*>(e->f);       // 2n floats
    float* save2 = reinterpret_cast<float*>(e->fd);     // 2n floats
    if (ens_cuda(e, cudaMemcpyAsync(save, e->x[0], 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune save") ||
        ens_cuda(e, cudaMemcpyAsync(save + n, e->x[1], 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune save") ||
        ens_cuda(e, cudaMemcpyAsync(save2, e->p[0], 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune save") ||
        ens_cuda(e, cudaMemcpyAsync(save2 + n, e->p[1], 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune save"))
        return IEGPU_ECUDA;
    e->mat = 0;
    std::vector<SplitCtl> ctl0(e->ctl_h, e->ctl_h + e->count);
    std::vector<int> cur0(e->cur_h, e->cur_h + e->count);
    std::vector<iegpu_bg> b((size_t)e->count);
    for (size_t ci = 0; ci < e->cls.size(); ++ci) {
        EnsClass& c = e->cls[ci];
        double best = 1e300;
        int3 pick = make_int3(c.TJ, c.PF, c.chunks);
        for (const int3& q : ens_candidates(e, c.N, (int)c.lats.size())) {
            c.TJ = q.x;
            c.PF = q.y;
            c.chunks = q.z;
            if (int rc = ens_layout(e)) return rc;
            for (int k = 0; k < e->count; ++k) b[(size_t)k] = bg0[k];
            double ms[2];
            int rc = ens_profile(e, nullptr, 4, b.data(), ms, (int)ci);
            // restore
            std::copy(ctl0.begin(), ctl0.end(), e->ctl_h);
            std::copy(cur0.begin(), cur0.end(), e->cur_h);
            if (ens_cuda(e, cudaMemcpyAsync(e->x[0], save, 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune restore") ||
                ens_cuda(e, cudaMemcpyAsync(e->x[1], save + n, 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune restore") ||
                ens_cuda(e, cudaMemcpyAsync(e->p[0], save2, 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune restore") ||
                ens_cuda(e, cudaMemcpyAsync(e->p[1], save2 + n, 4 * n, cudaMemcpyDeviceToDevice, e->stream), "tune restore"))
                return IEGPU_ECUDA;
            if (rc) return rc;
            if (ms[1] < best) { best = ms[1]; pick = q; }
        }
        c.TJ = pick.x;
        c.PF = pick.y;
        c.chunks = pick.z;
    }
    e->tuned = 1;
    if (int rc = ens_layout(e)) return rc;
    if (int rc = ens_upload_ctl(e)) return rc;
    return ens_sync(e, "autotune");
}

// ---- persistent mode -------------------------------------------------------

static constexpr int kEnsPersistSteps = 64;   // steps per cooperative launch

static bool ens_persist_ok(const iegpu_ens* e) {
    for (int N : e->sizes)
        if (N != 32 && N != 64 && N != 128) return false;
    return true;
}

// Plane chunks of a lattice in the persistent mode: 32 planes per item.
static int ens_persist_chunks(int N) { return N / 32; }

// Shapes of the persistent mode (8-row tiles, 2 planes ahead, 32 planes per
// item), the layout, the grid (every CTA resident) and the shared memory.
static int ens_persist_setup(iegpu_ens* e) {
    for (EnsClass& c : e->cls) {
        c.TJ = kEnsPersistTJ;
        c.PF = kEnsPersistPF;
        c.chunks = ens_persist_chunks(c.N);
    }
    if (int rc = ens_layout(e)) return rc;
    size_t smem = 0;
    for (int N : e->sizes) smem = std::max(smem, sizeof(float) * (size_t)split_row_smem_floats(kEnsPersistTJ, N, kEnsPersistPF));
    const void* fn = e->helper[0]->pot.table ? (const void*)k_ens_persist<true> : (const void*)k_ens_persist<false>;
    if (int rc = ens_cuda(e, smem_optin(fn, smem), "shared memory attribute")) return rc;
    int per_sm = 0;
    if (int rc = ens_cuda(e, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (kEnsPersistTJ + 1) * 32, smem),
                          "occupancy"))
        return rc;
    if (per_sm < 1) return ens_error(e, IEGPU_EUNSUPPORTED, "the persistent ensemble kernel does not fit an SM");
    e->persist_grid = per_sm * e->sms;
    e->persist_smem = smem;
    e->tuned = 1;
    return IEGPU_OK;
}

// One step's queue over the lattices with active[b]: every tile of every
// lattice, the largest lattices first (their items then come early in each
// step, and a step's items of a lattice long before its next step's).
static int ens_persist_queue(iegpu_ens* e, const std::vector<char>& active) {
    std::vector<int2> q;
    for (size_t ci = e->cls.size(); ci-- > 0;)
        for (int b : e->cls[ci].lats)
            if (active[(size_t)b])
                for (int t = 0; t < e->lat_h[(size_t)b].tiles; ++t) q.push_back(make_int2(b, t));
    if ((int)q.size() > e->queue_cap) {
        if (int rc = ens_sync(e, "queue")) return rc;
        if (e->queue) cudaFree(e->queue);
        e->queue = nullptr;
        e->queue_cap = 0;
        if (int rc = ens_alloc(e, &e->queue, q.size())) return rc;
        e->queue_cap = (int)q.size();
    }
    e->nqueue = (int)q.size();
    if (q.empty()) return IEGPU_OK;
    return ens_cuda(e, cudaMemcpyAsync(e->queue, q.data(), sizeof(int2) * q.size(), cudaMemcpyHostToDevice, e->stream),
                    "queue");
}

static int ens_persist_launch(iegpu_ens* e, int nsteps) {
    const EnsArgs A = ens_args(e);
    const size_t words = 2 + (size_t)e->count;
    if (int rc = ens_cuda(e, cudaMemsetAsync(e->qsync, 0, sizeof(unsigned) * words, e->stream), "queue reset")) return rc;
    if (int rc = ens_cuda(e, cudaMemsetAsync(e->counter, 0, sizeof(unsigned) * (size_t)e->count, e->stream),
                          "counter reset"))
        return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)e->persist_grid);
    cfg.blockDim = dim3((kEnsPersistTJ + 1) * 32);
    cfg.dynamicSmemBytes = e->persist_smem;
    cfg.stream = e->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const unsigned polls = 1u << 20;
    const cudaError_t err = A.P.table
        ? cudaLaunchKernelEx(&cfg, k_ens_persist<true>, A, (const int2*)e->queue, e->nqueue, nsteps, e->qsync, polls)
        : cudaLaunchKernelEx(&cfg, k_ens_persist<false>, A, (const int2*)e->queue, e->nqueue, nsteps, e->qsync, polls);
    e->launches++;
    return ens_cuda(e, err, "persistent ensemble launch");
}

static int ens_leapfrog_persist(iegpu_ens* e, const double* af, int max_steps, iegpu_bg* bg, int* steps) {
    e->mat = 0;
    bool shaped = e->persist_grid != 0;
    for (const EnsClass& c : e->cls)
        shaped = shaped && c.TJ == kEnsPersistTJ && c.PF == kEnsPersistPF && c.chunks == ens_persist_chunks(c.N);
    if (!shaped)
        if (int rc = ens_persist_setup(e)) return rc;
    ens_fill(e, bg, af, max_steps);
    if (int rc = ens_upload_ctl(e)) return rc;
    std::vector<char> active((size_t)e->count, 1);
    if (int rc = ens_persist_queue(e, active)) return rc;
    ens_launch_prime(e);
    int* seen = e->cur_h + e->count;
    long long launched = 0;
    int rc = IEGPU_OK;
    while (!rc && launched < max_steps && e->nqueue > 0) {
        const int n = (int)std::min<long long>(kEnsPersistSteps, max_steps - launched);
        if ((rc = ens_persist_launch(e, n))) break;
        launched += n;
        if ((rc = ens_cuda(e, cudaMemcpyAsync(seen, e->cur, sizeof(int) * (size_t)e->count, cudaMemcpyDeviceToHost,
                                              e->stream), "state copy")))
            break;
        if ((rc = ens_sync(e, "persistent ensemble step"))) break;
        int alive = 0, dead = 0;
        for (int b = 0; b < e->count; ++b) {
            if ((seen[b] & 2) == 0) alive++;
            else if (active[(size_t)b]) dead++;
        }
        if (alive == 0) break;
        if (dead > 0) {
            // drop the stopped lattices from the queue
            for (int b = 0; b < e->count; ++b) active[(size_t)b] = (seen[b] & 2) == 0;
            if ((rc = ens_persist_queue(e, active))) break;
        }
    }
    // the one-launch-per-step kernels and the priming reduction expect zeroed counters
    const int rc2 = ens_cuda(e, cudaMemsetAsync(e->counter, 0, sizeof(unsigned) * (size_t)e->count, e->stream),
                             "counter reset");
    if (rc) return rc;
    if (rc2) return rc2;
    if (int r = ens_finish(e, bg, steps)) return r;
    for (int b = 0; b < e->count; ++b)
        if (e->ctl_h[b].error == IEGPU_ETIMEOUT)
            return ens_error(e, IEGPU_ETIMEOUT, "a wait of the persistent ensemble kernel gave up (lattice %d)", b);
    return IEGPU_OK;
}

static int ens_leapfrog(iegpu_ens* e, const double* af, int max_steps, iegpu_bg* bg, int* steps) {
    if (steps)
        for (int b = 0; b < e->count; ++b) steps[b] = 0;
    if (max_steps < 0) return ens_error(e, IEGPU_EINVAL, "max_steps must be >= 0");
    if (max_steps == 0) return IEGPU_OK;
    if (e->persist) return ens_leapfrog_persist(e, af, max_steps, bg, steps);
    if (!e->tuned)
        if (int rc = ens_autotune(e, bg)) return rc;
    e->mat = 0;
    ens_fill(e, bg, af, max_steps);
    if (int rc = ens_upload_ctl(e)) return rc;
    std::vector<char> active((size_t)e->count, 1);
    if (int rc = ens_work(e, active)) return rc;
    ens_launch_prime(e);
    if (!ens_graph_current(e))
        if (int rc = ens_build_graph(e)) return rc;
    // graphs are queued one ahead of the host's check of the per-lattice words
    int* seen = e->cur_h + e->count;   // second half of the pinned mirror
    long long launched = 0;
    auto launch = [&]() -> int {
        if (int rc = ens_cuda(e, cudaGraphLaunch(e->exec, e->stream), "graph launch")) return rc;
        for (const EnsClass& c : e->cls)
            if (c.nwork) e->launches += e->graph_steps;
        launched += e->graph_steps;
        if (int rc = ens_cuda(e, cudaMemcpyAsync(seen, e->cur, sizeof(int) * (size_t)e->count, cudaMemcpyDeviceToHost,
                                                 e->stream), "state copy"))
            return rc;
        return ens_cuda(e, cudaEventRecord(e->ev[0], e->stream), "event");
    };
    if (int rc = launch()) return rc;
    while (true) {
        if (int rc = ens_cuda(e, cudaEventSynchronize(e->ev[0]), "step sync")) return rc;
        int alive = 0;
        bool compact = false;
        for (const EnsClass& c : e->cls) {
            int dead_tiles = 0;
            for (int b : c.lats) {
                const bool done = (seen[b] & 2) != 0;
                if (!done) alive++;
                else if (active[(size_t)b]) dead_tiles += e->lat_h[(size_t)b].tiles;
            }
            if (c.nwork > 0 && dead_tiles * 8 >= c.nwork) compact = true;
        }
        if (alive == 0 || launched >= max_steps) break;
        if (compact) {
            // drop the stopped lattices from the work tables
            for (int b = 0; b < e->count; ++b) active[(size_t)b] = (seen[b] & 2) == 0;
            if (int rc = ens_sync(e, "compaction")) return rc;
            if (int rc = ens_work(e, active)) return rc;
            if (int rc = ens_build_graph(e)) return rc;
        }
        if (int rc = launch()) return rc;
    }
    return ens_finish(e, bg, steps);
}

}  // namespace iegpu

using namespace iegpu;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

int iegpu_ens_create(const iegpu_config* cfg, const int* Ns, int count, iegpu_ens** out) {
    if (!cfg || !Ns || !out || count <= 0) return IEGPU_EINVAL;
    *out = nullptr;
    if (cfg->form != IEGPU_FORM_SPLIT || cfg->sigw) return IEGPU_EUNSUPPORTED;
    for (int b = 0; b < count; ++b)
        if (Ns[b] < 32 || Ns[b] > 256 || (Ns[b] & (Ns[b] - 1))) return IEGPU_EINVAL;
    iegpu_ens* e = new (std::nothrow) iegpu_ens();
    if (!e) return IEGPU_ENOMEM;
    e->cfg = *cfg;
    e->count = count;
    e->N.assign(Ns, Ns + count);
    e->off.resize((size_t)count);
    for (int b = 0; b < count; ++b) {
        e->off[(size_t)b] = e->total;
        e->total += (long long)Ns[b] * Ns[b] * Ns[b];
        if (std::find(e->sizes.begin(), e->sizes.end(), Ns[b]) == e->sizes.end()) e->sizes.push_back(Ns[b]);
    }
    int rc = IEGPU_OK;
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        delete e;
        return IEGPU_ECUDA;
    }
    e->sms = prop.multiProcessorCount;
    for (int N : e->sizes) {
        iegpu_config c1 = *cfg;
        c1.N = N;
        iegpu_ctx* h = nullptr;
        if (!rc) rc = iegpu_create(&c1, &h);
        if (h) e->helper.push_back(h);
    }
    if (!rc) rc = ens_cuda(e, cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "stream create");
    const size_t n = (size_t)e->total;
    for (int q = 0; q < 2 && !rc; ++q) {
        rc = ens_alloc(e, &e->x[q], n);
        if (!rc) rc = ens_alloc(e, &e->p[q], n);
    }
    if (!rc) rc = ens_alloc(e, &e->f, n);
    if (!rc) rc = ens_alloc(e, &e->fd, n);
    if (!rc) rc = ens_alloc(e, &e->dn, n);
    if (!rc) rc = ens_alloc(e, &e->ctl, (size_t)count);
    if (!rc) rc = ens_alloc(e, &e->cur, (size_t)count);
    if (!rc) rc = ens_alloc(e, &e->lat, (size_t)count);
    if (!rc) rc = ens_alloc(e, &e->counter, (size_t)count);
    if (!rc) rc = ens_alloc(e, &e->qsync, 2 + (size_t)count);
    if (!rc) rc = ens_alloc(e, &e->dctl, 1);
    if (!rc) rc = ens_alloc(e, &e->dscr, 4 * (size_t)count + 64);
    if (!rc) rc = ens_alloc(e, &e->iscr, 4 * (size_t)count + 64);
    if (!rc) rc = ens_cuda(e, cudaMallocHost(&e->ctl_h, sizeof(SplitCtl) * (size_t)count), "pinned alloc");
    if (!rc) rc = ens_cuda(e, cudaMallocHost(&e->cur_h, sizeof(int) * 2 * (size_t)count), "pinned alloc");
    if (!rc) rc = ens_cuda(e, cudaMallocHost(&e->dscr_h, sizeof(double) * (4 * (size_t)count + 64)), "pinned alloc");
    for (int q = 0; q < 2 && !rc; ++q) rc = ens_cuda(e, cudaEventCreate(&e->ev[q]), "event create");
    if (!rc) rc = ens_cuda(e, cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming), "event create");
    // one class per size: default shape whole planes (N <= 64) or 8-row tiles, 32 planes per chunk
    e->cls_of.assign((size_t)count, 0);
    std::vector<int> sorted = e->sizes;
    std::sort(sorted.begin(), sorted.end());
    for (int N : sorted) {
        EnsClass c;
        c.N = N;
        c.TJ = N <= 64 ? N : 8;
        c.PF = 2;
        c.chunks = N / 32 > N / 8 ? N / 8 : (N / 32 < 1 ? 1 : N / 32);
        for (int b = 0; b < count; ++b)
            if (Ns[b] == N) {
                c.lats.push_back(b);
                e->cls_of[(size_t)b] = (int)e->cls.size();
            }
        e->cls.push_back(c);
    }
    for (EnsClass& c : e->cls) {
        if (!rc) rc = ens_cuda(e, cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking), "stream create");
        if (!rc) rc = ens_cuda(e, cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming), "event create");
    }
    if (!rc) {
        memset(e->ctl_h, 0, sizeof(SplitCtl) * (size_t)count);
        memset(e->cur_h, 0, sizeof(int) * 2 * (size_t)count);
        rc = ens_cuda(e, cudaMemsetAsync(e->counter, 0, sizeof(unsigned) * (size_t)count, e->stream), "memset");
        if (!rc) rc = ens_cuda(e, cudaMemsetAsync(e->ctl, 0, sizeof(SplitCtl) * (size_t)count, e->stream), "memset");
        if (!rc) rc = ens_cuda(e, cudaMemsetAsync(e->cur, 0, sizeof(int) * (size_t)count, e->stream), "memset");
        if (!rc) rc = ens_cuda(e, cudaMemsetAsync(e->x[0], 0, sizeof(float) * n, e->stream), "memset");
        if (!rc) rc = ens_cuda(e, cudaMemsetAsync(e->p[0], 0, sizeof(float) * n, e->stream), "memset");
    }
    if (!rc) rc = ens_layout(e);
    if (rc) {
        iegpu_ens_destroy(e);
        return rc;
    }
    *out = e;
    return IEGPU_OK;
}

int iegpu_ens_destroy(iegpu_ens* e) {
    if (!e) return IEGPU_EINVAL;
    if (e->stream) cudaStreamSynchronize(e->stream);
    ens_destroy_graph(e);
    for (iegpu_ctx* h : e->helper) iegpu_destroy(h);
    void* dev[] = {e->x[0], e->x[1], e->p[0], e->p[1], e->f, e->fd, e->dn, e->ctl, e->cur, e->lat,
                   e->pwork, e->part, e->counter, e->dscr, e->iscr, e->red, e->dctl, e->queue, e->qsync};
    for (void* q : dev)
        if (q) cudaFree(q);
    for (EnsClass& c : e->cls) {
        if (c.work) cudaFree(c.work);
        if (c.done) cudaEventDestroy(c.done);
        if (c.stream) cudaStreamDestroy(c.stream);
    }
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->ctl_h) cudaFreeHost(e->ctl_h);
    if (e->cur_h) cudaFreeHost(e->cur_h);
    if (e->dscr_h) cudaFreeHost(e->dscr_h);
    for (cudaEvent_t ev : e->ev)
        if (ev) cudaEventDestroy(ev);
    if (e->stream) cudaStreamDestroy(e->stream);
    cudaGetLastError();
    delete e;
    return IEGPU_OK;
}

const char* iegpu_ens_last_error(const iegpu_ens* e) { return e ? e->err.c_str() : "null ensemble"; }

long long iegpu_ens_launch_count(const iegpu_ens* e) {
    if (!e) return 0;
    long long n = e->launches;
    for (const iegpu_ctx* h : e->helper) n += h->launches;
    return n;
}

void* iegpu_ens_stream(iegpu_ens* e) { return e ? static_cast<void*>(e->stream) : nullptr; }

int iegpu_ens_set_table(iegpu_ens* e, const double* phi, const double* V, const double* dV, int n) {
    if (!e) return IEGPU_EINVAL;
    for (iegpu_ctx* h : e->helper) {
        const int rc = iegpu_set_table(h, phi, V, dV, n);
        if (rc) return ens_error(e, rc, "%s", iegpu_last_error(h));
    }
    return IEGPU_OK;
}

int iegpu_ens_bunch_davies(iegpu_ens* e, const int* seeds, double phi0, double dphi0, double hi_cut, double lo_cut,
                           double* hubble_init) {
    if (!e || !seeds || !hubble_init) return IEGPU_EINVAL;
    if (int rc = ens_sync(e, "initial conditions")) return rc;
    for (int b = 0; b < e->count; ++b) {
        iegpu_ctx* h = ens_helper(e, e->N[(size_t)b]);
        const int rc = iegpu_bunch_davies(h, seeds[b], phi0, dphi0, hi_cut, lo_cut, &hubble_init[b]);
        if (rc) return ens_error(e, rc, "lattice %d: %s", b, iegpu_last_error(h));
        const size_t n = h->gs;
        const long long o = e->off[(size_t)b];
        // on the helper's stream, so its next lattice cannot overwrite the source first
        if (ens_cuda(e, cudaMemcpyAsync(e->x[0] + o, h->sp[h->cur], 4 * n, cudaMemcpyDeviceToDevice, h->stream), "copy") ||
            ens_cuda(e, cudaMemcpyAsync(e->p[0] + o, h->spi[h->cur], 4 * n, cudaMemcpyDeviceToDevice, h->stream), "copy"))
            return IEGPU_ECUDA;
        SplitCtl& C = e->ctl_h[b];
        memset(&C, 0, sizeof C);
        C.phibar = h->sctl_h->phibar;
        C.pibar = h->sctl_h->pibar;
        e->cur_h[b] = 0;
    }
    for (iegpu_ctx* h : e->helper)
        if (int rc = ens_cuda(e, cudaStreamSynchronize(h->stream), "initial conditions")) return rc;
    e->mat = 0;
    if (int rc = ens_upload_ctl(e)) return rc;
    return ens_sync(e, "initial conditions");
}

int iegpu_ens_evolve_fields(iegpu_ens* e, const double* d, iegpu_bg* bg) {
    if (!e || !d || !bg) return IEGPU_EINVAL;
    for (int b = 0; b < e->count; ++b) {
        bg[b].t += d[b];
        e->dscr_h[b] = d[b];
    }
    if (int rc = ens_cuda(e, cudaMemcpyAsync(e->dscr, e->dscr_h, sizeof(double) * (size_t)e->count,
                                             cudaMemcpyHostToDevice, e->stream), "drift steps"))
        return rc;
    const EnsArgs A = ens_args(e);
    k_ens_drift<<<(unsigned)(e->total / 256), 256, 0, e->stream>>>(A, e->dscr, e->count);
    e->launches++;
    for (int b = 0; b < e->count; ++b) bg[b].a += d[b] * bg[b].ad;
    e->mat = 0;
    return ens_download_ctl(e);
}

int iegpu_ens_leapfrog(iegpu_ens* e, const double* af, int max_steps, iegpu_bg* bg, int* steps) {
    if (!e || !af || !bg) return IEGPU_EINVAL;
    return ens_leapfrog(e, af, max_steps, bg, steps);
}

int iegpu_ens_profile(iegpu_ens* e, int nsteps, iegpu_bg* bg, double* ms_prime, double* ms_steps) {
    if (!e || !bg || !ms_prime || !ms_steps || nsteps < 0) return IEGPU_EINVAL;
    if (!e->tuned)
        if (int rc = ens_autotune(e, bg)) return rc;
    double ms[2];
    const int rc = ens_profile(e, nullptr, nsteps, bg, ms, -1);
    *ms_prime = ms[0];
    *ms_steps = ms[1];
    return rc;
}

int iegpu_ens_shapes(iegpu_ens* e, int* rows, int* prefetch, int* chunks) {
    if (!e) return IEGPU_EINVAL;
    for (int b = 0; b < e->count; ++b) {
        const EnsClass& c = e->cls[(size_t)e->cls_of[(size_t)b]];
        if (rows) rows[b] = c.TJ;
        if (prefetch) prefetch[b] = c.PF;
        if (chunks) chunks[b] = c.chunks;
    }
    return IEGPU_OK;
}

int iegpu_ens_autotune(iegpu_ens* e, const iegpu_bg* bg, int* rows, int* prefetch, int* chunks) {
    if (!e || !bg) return IEGPU_EINVAL;
    if (int rc = ens_autotune(e, bg)) return rc;
    for (int b = 0; b < e->count; ++b) {
        const EnsClass& c = e->cls[(size_t)e->cls_of[(size_t)b]];
        if (rows) rows[b] = c.TJ;
        if (prefetch) prefetch[b] = c.PF;
        if (chunks) chunks[b] = c.chunks;
    }
    return IEGPU_OK;
}

int iegpu_ens_set_persistent(iegpu_ens* e, int on) {
    if (!e) return IEGPU_EINVAL;
    if (on && !ens_persist_ok(e))
        return ens_error(e, IEGPU_EUNSUPPORTED, "the persistent ensemble launch covers lattices of N = 32, 64, 128");
    e->persist = on != 0;
    e->persist_grid = 0;
    return IEGPU_OK;
}

int iegpu_ens_set_shape(iegpu_ens* e, int N, int rows, int prefetch, int chunks) {
    if (!e) return IEGPU_EINVAL;
    for (EnsClass& c : e->cls) {
        if (c.N != N) continue;
        if (!ens_shape_ok(N, rows, prefetch, chunks))
            return ens_error(e, IEGPU_EINVAL,
                             "shape: rows 4|8 with prefetch 1|2 (rows 4 and N >= 128 also 3|4), rows 16 "
                             "(128 <= N <= 256) with prefetch 1..3, or rows N (N <= 64, whole planes) with "
                             "prefetch 2|4; 1 <= chunks <= N/8");
        c.TJ = rows;
        c.PF = prefetch;
        c.chunks = chunks;
        e->tuned = 1;
        return ens_layout(e);
    }
    return ens_error(e, IEGPU_EINVAL, "no lattice of size %d", N);
}

int iegpu_ens_timer_start(iegpu_ens* e) {
    if (!e) return IEGPU_EINVAL;
    return ens_cuda(e, cudaEventRecord(e->ev[1], e->stream), "timer start");
}

int iegpu_ens_timer_stop(iegpu_ens* e, float* ms) {
    if (!e || !ms) return IEGPU_EINVAL;
    cudaEvent_t stop;
    if (int rc = ens_cuda(e, cudaEventCreate(&stop), "timer")) return rc;
    cudaEventRecord(stop, e->stream);
    int rc = ens_cuda(e, cudaEventSynchronize(stop), "timer sync");
    if (!rc) rc = ens_cuda(e, cudaEventElapsedTime(ms, e->ev[1], stop), "timer elapsed");
    cudaEventDestroy(stop);
    return rc;
}

// F and FD: phibar + dphi and pibar + dpi of lattice b (or the FP64 fields of
// the deltaN stage once it has begun); DELTAN: the deltaN map.
int iegpu_ens_download(iegpu_ens* e, int lattice, int field, double* host) {
    if (!e || !host || lattice < 0 || lattice >= e->count) return IEGPU_EINVAL;
    if (field != IEGPU_F && field != IEGPU_FD && field != IEGPU_DELTAN) return IEGPU_EINVAL;
    if (field != IEGPU_DELTAN && !e->mat)
        if (int rc = ens_materialize(e)) return rc;
    const double* src = field == IEGPU_F ? e->f : field == IEGPU_FD ? e->fd : e->dn;
    const long long o = e->off[(size_t)lattice];
    const size_t n = (size_t)e->N[(size_t)lattice] * e->N[(size_t)lattice] * e->N[(size_t)lattice];
    if (int rc = ens_cuda(e, cudaMemcpyAsync(host, src + o, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream),
                          "download"))
        return rc;
    return ens_sync(e, "download");
}

}  // extern "C"
