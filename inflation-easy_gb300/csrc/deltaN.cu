// deltaN.cu -- per-site deltaN integration of src/evolution.cpp:1004-1037.
//
// Every site evolves independently in e-fold time:
//   fd += dN * (-(3 - fd^2/2) * (fd + V'/V))              (evolve_derivsN)
//   if (site still before the end surface) { deltaN += dN; f += dN fd }
//                                                          (evolve_fieldsN)
// so a thread keeps (f, fd, deltaN) of its site in registers for the whole run
// and the lattice is read and written once per launch: 0 B of HBM traffic per
// site-step.  The global scalars (t, a, Ne) are advanced by the host with the
// reference's own additions.  Compiled with -fmad=false: the per-site
// arithmetic reproduces the reference bit for bit.
#include "iegpu_internal.cuh"
#include "pot.cuh"

namespace iegpu {

template <bool TABLE, int CRIT>
__global__ void __launch_bounds__(256) k_deltaN(double* __restrict__ f, double* __restrict__ fd, double* __restrict__ dn,
                                                PotDev P, DevCtl* ctl, long long gs, double d, int nsteps,
                                                double phiref, double Vref, int do_derivs, int do_fields) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= gs) return;
    double x = f[id], v = fd[id], n = dn[id];
    const double aref = fabs(phiref);
    bool oor = false, bad = false;
    int l = 1;
    if (TABLE) {
        l = table_bracket(P, x, &oor);
        bad |= oor;
    }
    for (int s = 0; s < nsteps; ++s) {
        if (do_derivs) {
            double ratio;
            if (TABLE) {
                // pot_ratio, src/potential.cpp:177-192 (table values, no 1/B^2)
                l = table_walk(P, x, l, &oor);
                bad |= oor;
                const double pot = table_interp(P, P.V, P.dyV, x, l);
                const double der = table_interp(P, P.dV, P.dydV, x, l);
                ratio = der / pot;
            } else {
                const double pot = (P.V0 * (1.0 - P.c1 * (x * x))) / P.B2;
                const double der = (P.c2 * x) / P.B2;
                ratio = der / pot;
            }
            v = v + d * (-(3.0 - 0.5 * (v * v)) * (v + ratio));
        }
        if (do_fields) {
            bool act;
            if (CRIT > 0) act = fabs(x) > aref;
            else if (CRIT < 0) act = fabs(x) < aref;
            else {
                bool o2;
                act = V_exact<TABLE>(P, x, &o2) > Vref;
                bad |= o2;
            }
            if (act) {
                n = n + d;
                x = x + d * v;
            }
        }
    }
    if (bad) flag_error(ctl, IEGPU_ERANGE, x);
    f[id] = x;
    fd[id] = v;
    dn[id] = n;
}

// initializeN(), src/initialize.cpp:219-232
template <bool TABLE>
__global__ void k_initN(const double* __restrict__ f, double* __restrict__ fd, double* __restrict__ dn, PotDev P,
                        DevCtl* ctl, long long gs, double apow) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= gs) return;
    bool oor;
    const double H_lat = sqrt(V_exact<TABLE>(P, f[id], &oor) / 3.0);
    if (TABLE && oor) flag_error(ctl, IEGPU_ERANGE, f[id]);
    fd[id] = fd[id] * apow / H_lat;
    dn[id] = 0.0;
}

int deltaN_init(iegpu_ctx* c, double a) {
    const double apow = pow(a, c->cfg.rescale_s - 1.0);
    const unsigned grid = (unsigned)((c->gs + 255) / 256);
    if (cudaMemsetAsync(&c->ctl->error, 0, sizeof(int), c->stream) != cudaSuccess) return IEGPU_ECUDA;
    if (c->pot.table) k_initN<true><<<grid, 256, 0, c->stream>>>(c->f[c->cur], c->fd, c->dn, c->pot, c->ctl, (long long)c->gs, apow);
    else k_initN<false><<<grid, 256, 0, c->stream>>>(c->f[c->cur], c->fd, c->dn, c->pot, c->ctl, (long long)c->gs, apow);
    c->launches++;
    return IEGPU_OK;
}

template <bool TABLE>
static void launch_dn(iegpu_ctx* c, unsigned grid, double d, int nsteps, double phiref, double Vref, int dd, int df) {
    const int crit = c->cfg.criterion;
    if (crit > 0)
        k_deltaN<TABLE, 1><<<grid, 256, 0, c->stream>>>(c->f[c->cur], c->fd, c->dn, c->pot, c->ctl, (long long)c->gs, d, nsteps, phiref, Vref, dd, df);
    else if (crit < 0)
        k_deltaN<TABLE, -1><<<grid, 256, 0, c->stream>>>(c->f[c->cur], c->fd, c->dn, c->pot, c->ctl, (long long)c->gs, d, nsteps, phiref, Vref, dd, df);
    else
        k_deltaN<TABLE, 0><<<grid, 256, 0, c->stream>>>(c->f[c->cur], c->fd, c->dn, c->pot, c->ctl, (long long)c->gs, d, nsteps, phiref, Vref, dd, df);
}

int deltaN_steps(iegpu_ctx* c, double dN, int nsteps, double phiref, int do_derivs, int do_fields) {
    const unsigned grid = (unsigned)((c->gs + 255) / 256);
    // potential(phiref) for the generic criterion, src/evolution.cpp:1028
    const double Vref = (c->cfg.criterion == 0) ? host_potential(c, phiref) : 0.0;
    // chunks keep each launch short (about 2^24 site-steps per SM-thread slot)
    const int chunk = 2000;
    for (int s0 = 0; s0 < nsteps; s0 += chunk) {
        const int ns = (nsteps - s0) < chunk ? (nsteps - s0) : chunk;
        if (c->pot.table) launch_dn<true>(c, grid, dN, ns, phiref, Vref, do_derivs, do_fields);
        else launch_dn<false>(c, grid, dN, ns, phiref, Vref, do_derivs, do_fields);
        c->launches++;
    }
    return IEGPU_OK;
}

}  // namespace iegpu
