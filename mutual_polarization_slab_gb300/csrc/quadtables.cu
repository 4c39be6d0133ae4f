// Closed-form real-space couplings of the dipole + quadrupole operator
// (Capacitance_Quadrupole/RealSpaceTable.m:171-378): field/quadrupole
// (rrr.S, Ir.S + Sr + rS, Ir.S) and gradient/quadrupole (Irr:Q, Q,
// Irr:Q + 2Q.rr + 2rr.Q, rrrr:Q).  Each table has the form of the dipole ones,
//   cE r^-pE [E+(r) e^{-xi^2 (r+2)^2} + E-(r) e^{-xi^2 (r-2)^2} + E0(r) e^{-xi^2 r^2}]
// + cF r^-pF [F+(r) erfc(xi (r+2)) + F-(r) erfc(xi (r-2)) + F0(r) erfc(xi r)]
// + [r < 2] reg(r),
// with the polynomials written out in powers of r (highest first) from the
// reference's expressions.
#include <math.h>

#include <initializer_list>

#include "common.cuh"

namespace mps {

struct QSpec {
    double cE, cF;
    int pE, pF;
    int nE, nF;
    double E[3][10];
    double F[3][11];
};

struct QSet {
    QSpec t[7];
};

static void qset(QSpec &T, double cE, int pE, std::initializer_list<double> ep, std::initializer_list<double> em,
                 std::initializer_list<double> e0, double cF, int pF, std::initializer_list<double> fp,
                 std::initializer_list<double> fm, std::initializer_list<double> f0, double e0scale = 1.0,
                 double f0scale = 1.0) {
    T.cE = cE;
    T.pE = pE;
    T.cF = cF;
    T.pF = pF;
    T.nE = (int)ep.size();
    T.nF = (int)fp.size();
    int i = 0;
    for (double v : ep) T.E[0][i++] = v;
    i = 0;
    for (double v : em) T.E[1][i++] = v;
    i = 0;
    for (double v : e0) T.E[2][i++] = v * e0scale;
    i = 0;
    for (double v : fp) T.F[0][i++] = v;
    i = 0;
    for (double v : fm) T.F[1][i++] = v;
    i = 0;
    for (double v : f0) T.F[2][i++] = v * f0scale;
}

static void build_quad_specs(double xi, QSet &S) {
    const double x2 = xi * xi, x4 = x2 * x2, x6 = x4 * x2, x8 = x4 * x4, x10 = x8 * x2;
    const double sp3 = pow(MPS_PI, 1.5);
    const double pi = MPS_PI;
    const double a = 45 - 120 * x2 + 192 * x4 - 512 * x6;
    const double b = 2 * (45 + 24 * x2 - 64 * x4 + 512 * x6);
    const double c38 = 3 - 8 * x2;
    // field_quad_1: rrr.S
    qset(S.t[0], 15.0 / (16384 * sp3 * pow(xi, 7)), 4,
         {-24 * x6, 48 * x6, -4 * x4 * (9 - 8 * x2), 8 * x4 * c38, 2 * x2 * (21 - 80 * x2 + 64 * x4),
          -4 * x2 * c38 * c38, -a, -b},
         {-24 * x6, -48 * x6, -4 * x4 * (9 - 8 * x2), -8 * x4 * c38, 2 * x2 * (21 - 80 * x2 + 64 * x4),
          4 * x2 * c38 * c38, -a, b},
         {48 * x6, 0, 8 * x4 * (9 - 32 * x2), 0, -4 * x2 * (21 - 128 * x2), 0, 2 * (45 - 480 * x2), 0},
         15.0 / (32768 * pi * x8), 4,
         {48 * x8, 0, 32 * x6 * c38, 0, -24 * x4 * (3 - 16 * x2), 0, 72 * x2 * (1 - 8 * x2), 0,
          -45 + 480 * x2 + 4096 * x8},
         {48 * x8, 0, 32 * x6 * c38, 0, -24 * x4 * (3 - 16 * x2), 0, 72 * x2 * (1 - 8 * x2), 0,
          -45 + 480 * x2 + 4096 * x8},
         {-48 * x8, 0, -32 * x6 * c38, 0, 24 * x4 * (3 - 16 * x2), 0, -72 * x2 * (1 - 8 * x2), 0, 45 - 480 * x2}, 1.0,
         2.0);
    // field_quad_2: Ir.S + Sr + rS
    qset(S.t[1], 3.0 / (16384 * sp3 * pow(xi, 7)), 4,
         {-40 * x6, 80 * x6, -20 * x4 * (11 - 24 * x2), 8 * x4 * (45 + 8 * x2), -2 * x2 * (45 - 80 * x2 + 64 * x4),
          -4 * x2 * (15 + 48 * x2 - 64 * x4), a, b},
         {-40 * x6, -80 * x6, -20 * x4 * (11 - 24 * x2), -8 * x4 * (45 + 8 * x2), -2 * x2 * (45 - 80 * x2 + 64 * x4),
          4 * x2 * (15 + 48 * x2 - 64 * x4), a, -b},
         {8 * x6, 0, 4 * x4 * (11 - 32 * x2), 0, 2 * x2 * (9 - 64 * x2), 0, -9 + 96 * x2, 0},
         3.0 / (32768 * pi * x8), 4,
         {80 * x8, 0, 160 * x6 * c38, -2048 * x8, 120 * x4 * (3 - 16 * x2), 0, -120 * x2 * (1 - 8 * x2), 0,
          45 - 480 * x2 - 4096 * x8},
         {80 * x8, 0, 160 * x6 * c38, 2048 * x8, 120 * x4 * (3 - 16 * x2), 0, -120 * x2 * (1 - 8 * x2), 0,
          45 - 480 * x2 - 4096 * x8},
         {-16 * x8, 0, -32 * x6 * c38, 0, -24 * x4 * (3 - 16 * x2), 0, 24 * x2 * (1 - 8 * x2), 0, -9 + 96 * x2}, 10.0,
         10.0);
    // field_quad_3: Ir.S
    qset(S.t[2], 5.0 / (1024 * sp3 * pow(xi, 5)), 2, {4 * x4, -8 * x4, 16 * x2 * (1 - 2 * x2), -24 * x2, 3, 6},
         {4 * x4, 8 * x4, 16 * x2 * (1 - 2 * x2), 24 * x2, 3, -6},
         {-8 * x4, 0, -32 * x2 * (1 - 3 * x2), 0, 2 * (-3 + 24 * x2), 0}, 5.0 / (2048 * pi * x6), 2,
         {-8 * x6, 0, -12 * x4 * c38, 128 * x6, -6 * x2 * (3 - 16 * x2), 0, 3 - 24 * x2},
         {-8 * x6, 0, -12 * x4 * c38, -128 * x6, -6 * x2 * (3 - 16 * x2), 0, 3 - 24 * x2},
         {16 * x6, 0, 24 * x4 * c38, 0, 12 * x2 * (3 - 16 * x2), 0, 2 * (-3 + 24 * x2)});
    // grad_quad_1: Irr:Q
    {
        const double p1[9] = {16 * x8, 0, 96 * x6 - 128 * x8, 0, 72 * x4 - 192 * x6 + 256 * x8, 0,
                              -(24 * x2 - 96 * x4 + 256 * x6), 0, 9 - 48 * x2 + 192 * x4};
        qset(S.t[3], 75.0 / (16384 * sp3 * pow(xi, 7)), 3,
             {8 * x6, -16 * x6, 44 * x4 - 32 * x6, -(72 * x4 - 64 * x6), 18 * x2 + 32 * x4, 12 * x2 - 64 * x4,
              -(9 + 24 * x2), -(18 - 48 * x2)},
             {8 * x6, 16 * x6, 44 * x4 - 32 * x6, 72 * x4 - 64 * x6, 18 * x2 + 32 * x4, -(12 * x2 - 64 * x4),
              -(9 + 24 * x2), 18 - 48 * x2},
             {8 * x6, 0, 44 * x4 - 64 * x6, 0, 18 * x2 - 64 * x4 + 128 * x6, 0, -9 + 48 * x2 - 192 * x4, 0},
             75.0 / (32768 * pi * x8), 3, {-p1[0], -p1[1], -p1[2], -p1[3], -p1[4], -p1[5], -p1[6], -p1[7], -p1[8]},
             {-p1[0], -p1[1], -p1[2], -p1[3], -p1[4], -p1[5], -p1[6], -p1[7], -p1[8]},
             {p1[0], p1[1], p1[2], p1[3], p1[4], p1[5], p1[6], p1[7], p1[8]}, -2.0, 2.0);
    }
    // grad_quad_2: Q
    {
        const double q0[11] = {288 * x10, 0, 3600 * x8 - 4800 * x10, 0, 10800 * x6 - 28800 * x8 + 38400 * x10, 0,
                               5400 * x4 - 21600 * x6 + 57600 * x8, 0, -(1350 * x2 - 7200 * x4 + 28800 * x6), 0,
                               405 - 2700 * x2 + 14400 * x4};
        const double qp5 = 49152 * x10, qp10 = q0[10] + 49152 * x10;
        const double e1 = 135 + 180 * x2 + 480 * x4 - 768 * x6 + 2048 * x8;
        const double e0 = 270 - 1080 * x2 - 192 * x4 + 512 * x6 - 4096 * x8;
        qset(S.t[4], 3.0 / (32768 * sp3 * pow(xi, 9)), 5,
             {-48 * x8, 96 * x8, -(576 * x6 - 608 * x8), 1056 * x6 - 1216 * x8, -(1536 * x4 - 2576 * x6 + 3968 * x8),
              2160 * x4 - 4320 * x6 - 256 * x8, -(360 * x2 + 360 * x4 + 640 * x6 - 512 * x8),
              -(360 * x2 - 1680 * x4 - 768 * x6 + 1024 * x8), e1, e0},
             {-48 * x8, -96 * x8, -(576 * x6 - 608 * x8), -(1056 * x6 - 1216 * x8),
              -(1536 * x4 - 2576 * x6 + 3968 * x8), -(2160 * x4 - 4320 * x6 - 256 * x8),
              -(360 * x2 + 360 * x4 + 640 * x6 - 512 * x8), 360 * x2 - 1680 * x4 - 768 * x6 + 1024 * x8, e1, -e0},
             {144 * x8, 0, 1728 * x6 - 2400 * x8, 0, 4608 * x4 - 13200 * x6 + 19200 * x8, 0,
              1080 * x2 - 5400 * x4 + 19200 * x6, 0, -405 + 2700 * x2 - 14400 * x4, 0},
             1.0 / (65536 * pi * x10), 5, {q0[0], q0[1], q0[2], q0[3], q0[4], qp5, q0[6], q0[7], q0[8], q0[9], qp10},
             {q0[0], q0[1], q0[2], q0[3], q0[4], -qp5, q0[6], q0[7], q0[8], q0[9], qp10},
             {q0[0], q0[1], q0[2], q0[3], q0[4], q0[5], q0[6], q0[7], q0[8], q0[9], q0[10]}, 2.0 / 3.0, -2.0);
    }
    // grad_quad_3: Irr:Q + 2Q.rr + 2rr.Q
    {
        const double g1 = 135 + 180 * x2 + 480 * x4 - 768 * x6 + 2048 * x8;
        const double g0 = -270 + 1080 * x2 + 192 * x4 - 512 * x6 + 4096 * x8;
        const double rr[11] = {-96 * x10, 0, -720 * x8 + 960 * x10, 0, -(720 * x6 - 1920 * x8 + 2560 * x10), 0,
                               360 * x4 - 1440 * x6 + 3840 * x8, 0, -(270 * x2 - 1440 * x4 + 5760 * x6), 0,
                               135 - 900 * x2 + 4800 * x4 + 16384 * x10};
        const double ss[11] = {96 * x10, 0, 720 * x8 - 960 * x10, 0, 720 * x6 - 1920 * x8 + 2560 * x10, 0,
                               -(360 * x4 - 1440 * x6 + 3840 * x8), 0, 270 * x2 - 1440 * x4 + 5760 * x6, 0,
                               -135 + 900 * x2 - 4800 * x4};
        qset(S.t[5], -15.0 / (65536 * sp3 * pow(xi, 9)), 5,
             {48 * x8, -96 * x8, 336 * x6 - 288 * x8, -576 * (x6 - x8), 216 * x4 + 144 * x6 + 128 * x8,
              -(480 * x6 + 256 * x8), -(180 * x2 - 120 * x4 + 640 * x6 - 512 * x8), 720 * x4 + 768 * x6 - 1024 * x8,
              g1, -g0},
             {48 * x8, 96 * x8, 336 * x6 - 288 * x8, 576 * (x6 - x8), 216 * x4 + 144 * x6 + 128 * x8,
              480 * x6 + 256 * x8, -(180 * x2 - 120 * x4 + 640 * x6 - 512 * x8), -(720 * x4 + 768 * x6 - 1024 * x8),
              g1, g0},
             {48 * x8, 0, 336 * x6 - 480 * x8, 0, 216 * x4 - 720 * x6 + 1280 * x8, 0,
              -(180 * x2 - 840 * x4 + 2560 * x6), 0, 135 - 900 * x2 + 4800 * x4, 0},
             -15.0 / (131072 * pi * x10), 5,
             {rr[0], rr[1], rr[2], rr[3], rr[4], rr[5], rr[6], rr[7], rr[8], rr[9], rr[10]},
             {rr[0], rr[1], rr[2], rr[3], rr[4], rr[5], rr[6], rr[7], rr[8], rr[9], rr[10]},
             {ss[0], ss[1], ss[2], ss[3], ss[4], ss[5], ss[6], ss[7], ss[8], ss[9], ss[10]}, -2.0, 2.0);
    }
    // grad_quad_4: rrrr:Q
    {
        const double h1 = 945 + 1260 * x2 + 3360 * x4 - 5376 * x6 + 14336 * x8;
        const double h0 = 1890 - 7560 * x2 - 1344 * x4 + 3584 * x6 - 28672 * x8;
        const double tt[11] = {288 * x10, 0, 720 * x8 - 960 * x10, 0, -(720 * x6 - 1920 * x8 + 2560 * x10), 0,
                               1080 * x4 - 4320 * x6 + 11520 * x8, 0, -(1350 * x2 - 7200 * x4 + 28800 * x6), 0,
                               945 - 6300 * x2 + 33600 * x4 + 114688 * x10};
        const double uu10 = 945 - 6300 * x2 + 33600 * x4;
        qset(S.t[6], -15.0 / (65536 * sp3 * pow(xi, 9)), 5,
             {144 * x8, -288 * x8, 288 * x6 + 96 * x8, -(288 * x6 + 192 * x8), -(432 * x4 - 912 * x6 + 896 * x8),
              720 * x4 - 480 * x6 + 1792 * x8, 720 * x2 - 2280 * x4 + 4480 * x6 - 3584 * x8,
              -(1080 * x2 + 2160 * x4 + 5376 * x6 - 7168 * x8), -h1, -h0},
             {144 * x8, 288 * x8, 288 * x6 + 96 * x8, 288 * x6 + 192 * x8, -(432 * x4 - 912 * x6 + 896 * x8),
              -(720 * x4 - 480 * x6 + 1792 * x8), 720 * x2 - 2280 * x4 + 4480 * x6 - 3584 * x8,
              1080 * x2 + 2160 * x4 + 5376 * x6 - 7168 * x8, -h1, h0},
             {144 * x8, 0, 288 * x6 - 480 * x8, 0, -(432 * x4 - 1200 * x6 + 1280 * x8), 0,
              720 * x2 - 3000 * x4 + 6400 * x6, 0, -945 + 6300 * x2 - 33600 * x4, 0},
             15.0 / (131072 * pi * x10), 5,
             {tt[0], tt[1], tt[2], tt[3], tt[4], tt[5], tt[6], tt[7], tt[8], tt[9], tt[10]},
             {tt[0], tt[1], tt[2], tt[3], tt[4], tt[5], tt[6], tt[7], tt[8], tt[9], tt[10]},
             {tt[0], tt[1], tt[2], tt[3], tt[4], tt[5], tt[6], tt[7], tt[8], tt[9], uu10}, -2.0, -2.0);
    }
}

__device__ __forceinline__ double qhorner(const double *c, int nc, double r) {
    double v = c[0];
    for (int i = 1; i < nc; ++i) v = v * r + c[i];
    return v;
}

// Overlap corrections for r < 2.
__device__ double quad_overlap(int t, double r) {
    const double pi = MPS_PI;
    const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r4 * r;
    switch (t) {
        case 0: return -15.0 / (4 * pi * r4) + 15 * r2 / (64 * pi) * (1 - 3 * r2 / 16);
        case 1: return 3.0 / (4 * pi * r4) - 3 * r / (8 * pi) * (1 - 5 * r / 8 + 5 * r3 / 128);
        case 2: return 5 * r / (8 * pi) * (1 - 3 * r / 4 + r3 / 16);
        case 3: return 75 * r * (4 - r2) * (4 - r2) / (1024 * pi);
        case 4: return -3.0 / (2 * pi) * (1 / r5 - 1 + 25 * r / 32 - 25 * r3 / 256 + 3 * r5 / 512);
        case 5: {
            const double q = r2 - 4;
            return -15 * q * q * q * (3 * r4 + 6 * r2 + 8) / (2048 * pi * r5);
        }
        default: return -15 * (3584 - 80 * r4 * r2 - 30 * r4 * r4 + 9 * r5 * r5) / (2048 * pi * r5);
    }
}

// overlap = 0: no r < 2 overlap polynomial (Compute_Field_Quadrupole/RealSpaceTable.m comments them all out).
__global__ void k_quad_tables(const double *__restrict__ r, int64_t n, double xi, QSet S, double self_gq2,
                              int overlap, double *__restrict__ out) {
    const int64_t row = n + 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i == 0) {
            for (int t = 0; t < 7; ++t) out[t * row] = t == 4 ? self_gq2 : 0.0;
            continue;
        }
        const double rv = r[i - 1];
        const double ep = exp(-(rv + 2.0) * (rv + 2.0) * xi * xi);
        const double em = exp(-(rv - 2.0) * (rv - 2.0) * xi * xi);
        const double e0 = exp(-rv * rv * xi * xi);
        const double fp = erfc((rv + 2.0) * xi);
        const double fm = erfc((rv - 2.0) * xi);
        const double f0 = erfc(rv * xi);
        for (int t = 0; t < 7; ++t) {
            const QSpec &T = S.t[t];
            double v = T.cE / pow(rv, (double)T.pE) *
                       (qhorner(T.E[0], T.nE, rv) * ep + qhorner(T.E[1], T.nE, rv) * em +
                        qhorner(T.E[2], T.nE, rv) * e0);
            v += T.cF / pow(rv, (double)T.pF) *
                 (qhorner(T.F[0], T.nF, rv) * fp + qhorner(T.F[1], T.nF, rv) * fm + qhorner(T.F[2], T.nF, rv) * f0);
            if (rv < 2.0 && overlap) v += quad_overlap(t, rv);
            out[t * row + i] = v;
        }
    }
}

// grad_quad_2 at r = 0 (CQ/RealSpaceTable.m:373-375).
static double quad_self_value(double xi) {
    const double x2 = xi * xi, x4 = x2 * x2, x5 = x4 * xi;
    const double e4 = exp(-4 * x2);
    return 1.0 / (2 * MPS_PI) *
           (3 * (3 - 10 * x2 + 20 * x4) / (8 * sqrt(MPS_PI) * x5) - 3 * (3 + 2 * x2 + 4 * x4) * e4 / (8 * sqrt(MPS_PI) * x5) +
            3 * erfc(2 * xi));
}

}  // namespace mps

using namespace mps;

extern "C" int mps_quad_table(const double *r, int64_t n, double xi, double *tables, mps_stream_t stream) {
    if (n < 0 || !tables || (n > 0 && !r) || !(xi > 0)) return MPS_BAD_ARG;
    QSet S;
    build_quad_specs(xi, S);
    cudaStream_t s = (cudaStream_t)stream;
    k_quad_tables<<<grid_for(n + 1, 256), 256, 0, s>>>(r, n, xi, S, quad_self_value(xi), 1, tables);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

extern "C" int mps_quad_table_probe(const double *r, int64_t n, double xi, double *tables, mps_stream_t stream) {
    if (n < 0 || !tables || (n > 0 && !r) || !(xi > 0)) return MPS_BAD_ARG;
    QSet S;
    build_quad_specs(xi, S);
    cudaStream_t s = (cudaStream_t)stream;
    k_quad_tables<<<grid_for(n + 1, 256), 256, 0, s>>>(r, n, xi, S, quad_self_value(xi), 0, tables);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}
