// ensemble.cuh -- an ensemble of independent lattices (seeds, sizes) held in
// one set of device buffers and evolved together in the split form.
//
// Device layout: the lattices are concatenated, lattice b occupying sites
// [off_b, off_b + N_b^3) of every per-site array, each in the one-lattice
// layout (k fastest).  Per-site arrays:
//   x[2], p[2]      dphi, dpi (FP32 ping-pong; cur[b] & 1 says which half is current)
//   f, fd, dn       FP64 field, velocity and deltaN for the deltaN stage
// Per lattice: a SplitCtl (its own a, ad, t, phibar, pibar, step
// coefficients, stop condition), a reduction counter, partial-sum slots and
// the word cur[b] (bit 0: current half; bit 1: the lattice has stopped).
// Every N^3 here is a multiple of 256, so a 256-thread block of a per-site
// kernel never straddles two lattices.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "iegpu_internal.cuh"

namespace iegpu {

struct EnsLat {
    long long off;   // first site of the lattice
    int lg;          // log2 N
    int rowtiles;    // N / rows per tile of the step kernel
    int chunks;      // plane chunks of the step kernel
    int tiles;       // rowtiles * chunks: CTAs of one step
    int pslots;      // CTAs of the priming reduction
    int part_off;    // first partial slot (3 doubles per slot)
    SplitConst K;
};

// Lattice holding site `site` (binary search over the offsets).
__device__ __forceinline__ int ens_lattice_of(const EnsLat* lat, int count, long long site) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (lat[mid].off <= site) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The lattices of one size, stepped by one kernel per step on their own
// stream (the classes run side by side as parallel branches of the graph).
struct EnsClass {
    int N = 0;
    std::vector<int> lats;
    int TJ = 8, PF = 2, chunks = 1;   // rows per tile (TJ == N: whole planes), planes prefetched
    int2* work = nullptr;             // (lattice, tile) of every CTA
    int work_cap = 0;
    int nwork = 0;
    int graph_nwork = -1;
    size_t smem = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

}  // namespace iegpu

struct iegpu_ens {
    iegpu_config cfg;
    int count = 0;
    std::vector<int> N;
    std::vector<long long> off;
    long long total = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    long long launches = 0;

    // one single-lattice split context per distinct N: initial conditions,
    // FFT-based spectra and the table live there
    std::vector<int> sizes;
    std::vector<iegpu_ctx*> helper;

    float* x[2] = {nullptr, nullptr};
    float* p[2] = {nullptr, nullptr};
    double* f = nullptr;
    double* fd = nullptr;
    double* dn = nullptr;
    iegpu::SplitCtl* ctl = nullptr;
    iegpu::SplitCtl* ctl_h = nullptr;   // pinned mirror
    int* cur = nullptr;
    int* cur_h = nullptr;                // pinned mirror
    iegpu::EnsLat* lat = nullptr;
    std::vector<iegpu::EnsLat> lat_h;
    std::vector<iegpu::EnsClass> cls;    // one per distinct N, ascending
    std::vector<int> cls_of;             // class of every lattice
    int2* pwork = nullptr;               // (lattice, slot) of every priming CTA
    int npwork = 0;
    double* part = nullptr;              // partial sums, 3 doubles per slot
    size_t part_cap = 0;
    unsigned* counter = nullptr;
    double* dscr = nullptr;              // per-lattice scalars of a call (count doubles x 4)
    double* dscr_h = nullptr;            // pinned mirror
    int* iscr = nullptr;                 // per-lattice integer results (count x 4)
    double* red = nullptr;               // reduction scratch
    size_t red_cap = 0;
    int mat = 0;                         // the FP64 arrays hold the fields (deltaN stage)
    iegpu::DevCtl* dctl = nullptr;       // error word of the deltaN kernels
    // results of the deltaN stage, per lattice
    int zeta_ready = 0;
    double zeta_cutoff = 0.0;            // Nend - dN
    std::vector<float> nmean;
    std::vector<double> phiref;

    int tuned = 0;
    // persistent mode: one cooperative launch of up to kEnsPersistSteps steps
    // over a queue of (lattice, tile) items of every size, big lattices first
    int persist = 0;
    int2* queue = nullptr;               // one step's items
    int queue_cap = 0;
    int nqueue = 0;
    unsigned* qsync = nullptr;           // [0] claim counter, [1] abort flag, then the per-lattice published steps
    int persist_grid = 0;
    size_t persist_smem = 0;
    cudaGraphExec_t exec = nullptr;
    int graph_steps = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaEvent_t fork = nullptr;
};

namespace iegpu {

int ens_error(iegpu_ens* e, int code, const char* fmt, ...);
int ens_cuda(iegpu_ens* e, cudaError_t err, const char* what);

// ensemble_dn.cu (the FP64 deltaN stage, compiled without contractions)
int ens_materialize(iegpu_ens* e);
int ens_initN(iegpu_ens* e, const double* apow_h);
int ens_deltaN_steps(iegpu_ens* e, double d, int nsteps, const double* phiref_h, int do_derivs, int do_fields);
int ens_phiref(iegpu_ens* e, double* phiref_h);
int ens_saveN_mean(iegpu_ens* e, double cutoff, float* nmean_h);
int ens_shift(iegpu_ens* e, const float* nmean_h);
int ens_zeta_moments(iegpu_ens* e, int N, double* sum, double* sumsq, long long* n);
int ens_zeta_hist(iegpu_ens* e, int N, double lo, double width, int nbins, long long* counts, long long* outside);

}  // namespace iegpu
