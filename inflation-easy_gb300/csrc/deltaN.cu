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
//
// The RK4 and RK45 branches of the loop (deltaN_integrator = rk4 | rk45,
// src/evolution.cpp:1039-1267) are per site too: an RK4 step keeps its four
// stages in registers, so a launch runs many steps, and an RK45 attempt
// evaluates its seven stages, the 5th-order candidate and the site's error
// term in one pass, the error norm summed over the lattice in a fixed order.
#include <cstdio>

#include "iegpu_internal.cuh"
#include "pot.cuh"
#include "reduce.cuh"
#include "rk_tableau.cuh"

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
                const double pot = div_exact(P.V0 * (1.0 - P.c1 * (x * x)), P.divB2);
                const double der = div_exact(P.c2 * x, P.divB2);
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

// ---------------------------------------------------------------------------
// RK4 / RK45 branches of run_deltaN_loop
// ---------------------------------------------------------------------------

__constant__ double cRk4A[IE_RK_STAGES][IE_RK_STAGES] = IE_RK4_A_INIT;
__constant__ double cRk4B[IE_RK_STAGES] = IE_RK4_B_INIT;
__constant__ double cDpA[IE_RK_STAGES][IE_RK_STAGES] = IE_DP_A_INIT;
__constant__ double cDpB[IE_RK_STAGES] = IE_DP_B_INIT;
__constant__ double cDpE[IE_RK_STAGES] = IE_DP_E_INIT;
static const double hRk4B[IE_RK_STAGES] = IE_RK4_B_INIT;
static const double hDpB[IE_RK_STAGES] = IE_DP_B_INIT;
static const double hDpE[IE_RK_STAGES] = IE_DP_E_INIT;

// compute_deltaN_rhs at one site, src/evolution.cpp:1063-1113: V and V' as
// evaluate_potential_from_value gives them (each divided by B^2), k_fd =
// -(3 - fd^2/2)(fd + V'/V), and k_f = fd, k_dn = 1 at active sites (0, 0
// beyond the end surface).  l is the site's bracket, walked from the last.
template <bool TABLE, int CRIT>
__device__ __forceinline__ void rhsN(const PotDev& P, double x, double v, double aref, double Vref, int& l,
                                     bool& bad, double& kf, double& kfd, double& kdn) {
    double pot, dpot;
    if (TABLE) {
        bool oor;
        l = table_walk(P, x, l, &oor);
        bad |= oor;
        pot = div_exact(table_interp(P, P.V, P.dyV, x, l), P.divB2);
        dpot = div_exact(table_interp(P, P.dV, P.dydV, x, l), P.divB2);
    } else {
        pot = div_exact(P.V0 * (1.0 - P.c1 * (x * x)), P.divB2);
        dpot = div_exact(P.c2 * x, P.divB2);
    }
    const double ratio = dpot / pot;
    bool act;
    if (CRIT > 0) act = fabs(x) > aref;
    else if (CRIT < 0) act = fabs(x) < aref;
    else act = pot > Vref;
    kfd = -(3.0 - 0.5 * (v * v)) * (v + ratio);
    kf = act ? v : 0.0;
    kdn = act ? 1.0 : 0.0;
}

// nsteps of rk4_step_deltaN(h), src/evolution.cpp:1176-1188, per site in
// registers: stage states f + h sum_q A k_f, fd + h sum_q A k_fd (sums from
// 0.0 in stage order, zero coefficients skipped), then the weighted update of
// f, fd and deltaN.
template <bool TABLE, int CRIT>
__global__ void __launch_bounds__(256) k_deltaN_rk4(double* __restrict__ f, double* __restrict__ fd,
                                                    double* __restrict__ dn, PotDev P, DevCtl* ctl, long long gs,
                                                    double h, int nsteps, double phiref, double Vref) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= gs) return;
    double x = f[id], v = fd[id], n = dn[id];
    const double aref = fabs(phiref);
    bool bad = false;
    int l = 1;
    if (TABLE) {
        bool oor;
        l = table_bracket(P, x, &oor);
        bad |= oor;
    }
    for (int s = 0; s < nsteps; ++s) {
        double kf[4], kfd[4], kdn[4];
        rhsN<TABLE, CRIT>(P, x, v, aref, Vref, l, bad, kf[0], kfd[0], kdn[0]);
#pragma unroll
        for (int st = 1; st < 4; ++st) {
            double sf = 0.0, sfd = 0.0;
#pragma unroll
            for (int q = 0; q < st; ++q) {
                const double cq = cRk4A[st][q];
                if (cq == 0.0) continue;
                sf += cq * kf[q];
                sfd += cq * kfd[q];
            }
            rhsN<TABLE, CRIT>(P, x + h * sf, v + h * sfd, aref, Vref, l, bad, kf[st], kfd[st], kdn[st]);
        }
        double sf = 0.0, sfd = 0.0, sdn = 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double bq = cRk4B[q];
            if (bq == 0.0) continue;
            sf += bq * kf[q];
            sfd += bq * kfd[q];
            sdn += bq * kdn[q];
        }
        x += h * sf;
        v += h * sfd;
        n += h * sdn;
    }
    if (bad) flag_error(ctl, IEGPU_ERANGE, x);
    f[id] = x;
    fd[id] = v;
    dn[id] = n;
}

// One rk45_step_deltaN attempt, src/evolution.cpp:1190-1267, lattice part:
// per site the seven stages, the candidate y5 = y + sum_q h b_q k_q and the
// error sum_q h e_q k_q of f, fd and deltaN (terms added in stage order),
// the candidate into y5[0, gs, 2 gs), and the site's
// (err_f/s_f)^2 + (err_fd/s_fd)^2 + (err_dn/s_dn)^2, summed by the last CTA
// in a fixed order into sums[0].
template <bool TABLE, int CRIT>
__global__ void __launch_bounds__(256) k_deltaN_rk45(const double* __restrict__ f, const double* __restrict__ fd,
                                                     const double* __restrict__ dn, double* __restrict__ y5,
                                                     PotDev P, DevCtl* ctl, long long gs, double h, double phiref,
                                                     double Vref, double atol, double rtol, double* part,
                                                     unsigned* counter, double* sums) {
    const double aref = fabs(phiref);
    double acc[1] = {0.0};
    bool bad = false;
    double badval = 0.0;
    for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < gs;
         id += (long long)gridDim.x * blockDim.x) {
        const double x = f[id], v = fd[id], n = dn[id];
        int l = 1;
        bool b0 = false;
        if (TABLE) {
            bool oor;
            l = table_bracket(P, x, &oor);
            b0 |= oor;
        }
        double kf[IE_RK_STAGES], kfd[IE_RK_STAGES], kdn[IE_RK_STAGES];
        rhsN<TABLE, CRIT>(P, x, v, aref, Vref, l, b0, kf[0], kfd[0], kdn[0]);
#pragma unroll
        for (int st = 1; st < IE_RK_STAGES; ++st) {
            double sf = 0.0, sfd = 0.0;
#pragma unroll
            for (int q = 0; q < st; ++q) {
                const double cq = cDpA[st][q];
                if (cq == 0.0) continue;
                sf += cq * kf[q];
                sfd += cq * kfd[q];
            }
            rhsN<TABLE, CRIT>(P, x + h * sf, v + h * sfd, aref, Vref, l, b0, kf[st], kfd[st], kdn[st]);
        }
        double y5f = x, y5fd = v, y5dn = n, ef = 0.0, efd = 0.0, edn = 0.0;
#pragma unroll
        for (int q = 0; q < IE_RK_STAGES; ++q) {
            const double bq = cDpB[q], eq = cDpE[q];
            if (bq != 0.0) {
                y5f += h * bq * kf[q];
                y5fd += h * bq * kfd[q];
                y5dn += h * bq * kdn[q];
            }
            if (eq != 0.0) {
                ef += h * eq * kf[q];
                efd += h * eq * kfd[q];
                edn += h * eq * kdn[q];
            }
        }
        y5[id] = y5f;
        y5[gs + id] = y5fd;
        y5[2 * gs + id] = y5dn;
        const double sf = atol + rtol * (fabs(x) < fabs(y5f) ? fabs(y5f) : fabs(x));
        const double sfd = atol + rtol * (fabs(v) < fabs(y5fd) ? fabs(y5fd) : fabs(v));
        const double sdn = atol + rtol * (fabs(n) < fabs(y5dn) ? fabs(y5dn) : fabs(n));
        const double qf = ef / sf, qfd = efd / sfd, qdn = edn / sdn;
        acc[0] += qf * qf + qfd * qfd + qdn * qdn;
        if (b0 && !bad) {
            bad = true;
            badval = x;
        }
    }
    if (bad) flag_error(ctl, IEGPU_ERANGE, badval);
    block_sum<1>(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc[0];
    if (!arrive_last(counter)) return;
    if (threadIdx.x < 32) {
        double tot[1];
        sum_partials<1>(part, gridDim.x, tot);
        if (threadIdx.x == 0) {
            *counter = 0;
            sums[0] = tot[0];
        }
    }
}

template <bool TABLE>
static void launch_rk4N(iegpu_ctx* c, unsigned grid, double h, int nsteps, double phiref, double Vref) {
    double* f = c->f[c->cur];
    const long long gs = (long long)c->gs;
    const int crit = c->cfg.criterion;
    if (crit > 0) k_deltaN_rk4<TABLE, 1><<<grid, 256, 0, c->stream>>>(f, c->fd, c->dn, c->pot, c->ctl, gs, h, nsteps, phiref, Vref);
    else if (crit < 0) k_deltaN_rk4<TABLE, -1><<<grid, 256, 0, c->stream>>>(f, c->fd, c->dn, c->pot, c->ctl, gs, h, nsteps, phiref, Vref);
    else k_deltaN_rk4<TABLE, 0><<<grid, 256, 0, c->stream>>>(f, c->fd, c->dn, c->pot, c->ctl, gs, h, nsteps, phiref, Vref);
}

template <bool TABLE>
static void launch_rk45N(iegpu_ctx* c, double h, double phiref, double Vref, double atol, double rtol) {
    const double* f = c->f[c->cur];
    const long long gs = (long long)c->gs;
    const int crit = c->cfg.criterion;
    const unsigned g = (unsigned)c->red_grid;
    if (crit > 0)
        k_deltaN_rk45<TABLE, 1><<<g, 256, 0, c->stream>>>(f, c->fd, c->dn, c->dn_y5, c->pot, c->ctl, gs, h, phiref, Vref, atol, rtol, c->part, c->counter, c->misc);
    else if (crit < 0)
        k_deltaN_rk45<TABLE, -1><<<g, 256, 0, c->stream>>>(f, c->fd, c->dn, c->dn_y5, c->pot, c->ctl, gs, h, phiref, Vref, atol, rtol, c->part, c->counter, c->misc);
    else
        k_deltaN_rk45<TABLE, 0><<<g, 256, 0, c->stream>>>(f, c->fd, c->dn, c->dn_y5, c->pot, c->ctl, gs, h, phiref, Vref, atol, rtol, c->part, c->counter, c->misc);
}

static double Vref_of(const iegpu_ctx* c, double phiref) {
    // g_deltaN_phiref_potential = potential(phiref), src/evolution.cpp:1305
    return (c->cfg.criterion == 0) ? host_potential(c, phiref) : 0.0;
}

// nsteps of rk4_step_deltaN(h): the lattice on the device, then a and t as
// apply_deltaN_weighted_update advances them (a with its constant derivative
// ad).  The caller advances Ne.
int deltaN_rk4(iegpu_ctx* c, double h, int nsteps, double phiref, iegpu_bg* bg) {
    const unsigned grid = (unsigned)((c->gs + 255) / 256);
    const double Vref = Vref_of(c, phiref);
    const int chunk = 500;
    for (int s0 = 0; s0 < nsteps; s0 += chunk) {
        const int ns = (nsteps - s0) < chunk ? (nsteps - s0) : chunk;
        if (c->pot.table) launch_rk4N<true>(c, grid, h, ns, phiref, Vref);
        else launch_rk4N<false>(c, grid, h, ns, phiref, Vref);
        c->launches++;
    }
    for (int s = 0; s < nsteps; ++s) {
        for (int q = 0; q < 4; ++q) {
            const double bq = hRk4B[q];
            if (bq == 0.0) continue;
            bg->a += h * bq * bg->ad;
        }
        bg->t += h;
    }
    return IEGPU_OK;
}

static int dn_status(iegpu_ctx* c) {
    if (c->ctl_h->error) {
        double v = 0;
        cudaMemcpy(&v, &c->ctl->errval, sizeof(double), cudaMemcpyDeviceToHost);
        return set_error(c, IEGPU_ERANGE, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n", v,
                         c->htab_x.back(), c->htab_x.front());
    }
    return IEGPU_OK;
}

// rk45_step_deltaN(h, hmax, h_next): one attempt; on acceptance the
// candidate becomes the state, a = a5 and t += h.
static int rk45N_attempt(iegpu_ctx* c, const iegpu_rk45_controls& K, double h, double hmax, double phiref,
                         double Vref, double* h_next, int* accepted, iegpu_bg* bg) {
    if (c->pot.table) launch_rk45N<true>(c, h, phiref, Vref, K.abs_tol, K.rel_tol);
    else launch_rk45N<false>(c, h, phiref, Vref, K.abs_tol, K.rel_tol);
    c->launches++;
    if (check_cuda(c, cudaMemcpyAsync(c->misc_h, c->misc, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "deltaN RK45"))
        return IEGPU_ECUDA;
    if (check_cuda(c, cudaMemcpyAsync(&c->ctl_h->error, &c->ctl->error, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "deltaN RK45"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "deltaN RK45")) return IEGPU_ECUDA;
    if (int rc = dn_status(c)) return rc;
    double a5 = bg->a, erra = 0.0;
    for (int q = 0; q < IE_RK_STAGES; ++q) {
        if (hDpB[q] != 0.0) a5 += h * hDpB[q] * bg->ad;
        if (hDpE[q] != 0.0) erra += h * hDpE[q] * bg->ad;
    }
    double err_acc = c->misc_h[0];
    const size_t nvars = 3 * c->gs + 1;
    const double sa = K.abs_tol + K.rel_tol * (fabs(bg->a) < fabs(a5) ? fabs(a5) : fabs(bg->a));
    err_acc += (erra / sa) * (erra / sa);
    const double err_norm = sqrt(err_acc / (double)nvars);
    const double safe_err = err_norm < 1e-16 ? 1e-16 : err_norm;
    double factor = K.safety * pow(safe_err, -0.2);
    factor = (factor < 0.1) ? 0.1 : (5.0 < factor) ? 5.0 : factor;
    if (err_norm <= 1.0) {
        const size_t bytes = sizeof(double) * c->gs;
        cudaError_t e = cudaMemcpyAsync(c->f[c->cur], c->dn_y5, bytes, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->fd, c->dn_y5 + c->gs, bytes, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->dn, c->dn_y5 + 2 * c->gs, bytes, cudaMemcpyDeviceToDevice, c->stream);
        if (check_cuda(c, e, "deltaN RK45 accept")) return IEGPU_ECUDA;
        bg->a = a5;
        bg->t += h;
        *h_next = rk45_clamp(K, h * factor, hmax);
        *accepted = 1;
        return IEGPU_OK;
    }
    const double f2 = factor < 0.5 ? factor : 0.5;
    *h_next = rk45_clamp(K, h * (0.1 < f2 ? f2 : 0.1), hmax);
    *accepted = 0;
    return IEGPU_OK;
}

// The RK45 branch of run_deltaN_loop, src/evolution.cpp:1334-1367: while
// Ne <= Nend, hmax from dN, h clamped, attempts until one is accepted
// (rk45_accept_step), then Ne += h with the step proposed for the next
// iteration, as the reference adds it.
int deltaN_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double dN, double Nend, int max_steps, double phiref,
                double* h, double* Ne, iegpu_bg* bg, int* steps, double* Ne_trace) {
    if (steps) *steps = 0;
    if (!c->dn_y5) {
        if (cudaMalloc(&c->dn_y5, sizeof(double) * 3 * c->gs) != cudaSuccess) {
            cudaGetLastError();
            c->dn_y5 = nullptr;
            return set_error(c, IEGPU_ENOMEM, "device allocation of the deltaN RK45 candidate failed");
        }
    }
    const iegpu_rk45_controls K = rk45_sanitized(c, ctl);
    const double Vref = Vref_of(c, phiref);
    int n = 0;
    while (n < max_steps && *Ne <= Nend) {
        const double hmax = rk45_hmax(K, dN);
        *h = rk45_clamp(K, *h, hmax);
        int accepted = 0, attempts = 0;
        while (!accepted) {
            double hs = *h;
            if (int rc = rk45N_attempt(c, K, *h, hmax, phiref, Vref, &hs, &accepted, bg)) {
                if (steps) *steps = n;
                return rc;
            }
            *h = hs;
            ++attempts;
            if (!accepted && (attempts > 25 || *h <= K.min_dt * (1.0 + 1e-12))) {
                if (steps) *steps = n;
                return set_error(c, IEGPU_ECONVERGE, "RK45 failed to converge in deltaN loop at N=%e, t=%e (attempts=%d, h=%e)\n",
                                 *Ne, bg->t, attempts, *h);
            }
        }
        *Ne += *h;
        if (Ne_trace) Ne_trace[n] = *Ne;
        ++n;
    }
    if (steps) *steps = n;
    return sync_and_check(c, "deltaN RK45");
}

}  // namespace iegpu
