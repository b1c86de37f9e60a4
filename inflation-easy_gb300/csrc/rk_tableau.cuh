// rk_tableau.cuh -- Butcher tableaux of the Runge-Kutta integrators, as
// initialiser lists for the host tables (leapfrog_fp64.cu) and the __constant__
// tables of the per-site deltaN kernels (deltaN.cu).
//
// RK4_A, RK4_B (src/evolution.cpp:601-613) and the Dormand-Prince 5(4)
// coefficients of DormandPrince45Coefficients (:366-414, tables :615-637):
// the published values, with the embedded error weights e = b - b* formed
// from the two weight rows in double precision.  Rows are padded to seven
// stages; a zero entry is skipped where it is used, as the reference does.
#pragma once

#define IE_RK_STAGES 7

#define IE_DP_B1 (35.0 / 384.0)
#define IE_DP_B3 (500.0 / 1113.0)
#define IE_DP_B4 (125.0 / 192.0)
#define IE_DP_B5 (-2187.0 / 6784.0)
#define IE_DP_B6 (11.0 / 84.0)

#define IE_RK4_A_INIT {{0.0}, {0.5}, {0.0, 0.5}, {0.0, 0.0, 1.0}}
#define IE_RK4_B_INIT {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0}

#define IE_DP_A_INIT                                                                               \
    {{0.0},                                                                                        \
     {1.0 / 5.0},                                                                                  \
     {3.0 / 40.0, 9.0 / 40.0},                                                                     \
     {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0},                                                      \
     {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0},                       \
     {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0},           \
     {IE_DP_B1, 0.0, IE_DP_B3, IE_DP_B4, IE_DP_B5, IE_DP_B6}}
#define IE_DP_B_INIT {IE_DP_B1, 0.0, IE_DP_B3, IE_DP_B4, IE_DP_B5, IE_DP_B6, 0.0}
#define IE_DP_E_INIT                                                                               \
    {IE_DP_B1 - 5179.0 / 57600.0, 0.0, IE_DP_B3 - 7571.0 / 16695.0, IE_DP_B4 - 393.0 / 640.0,      \
     IE_DP_B5 - -92097.0 / 339200.0, IE_DP_B6 - 187.0 / 2100.0, -(1.0 / 40.0)}
