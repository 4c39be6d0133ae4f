// Hand-written mixed-radix 3-D real FFT pipeline with the dipole Green's scale
// fused into its z pass, in two arithmetics:
//   double-float (float hi + float lo, ~48-bit significand) for the
//   float64-accurate matvec of the refinement residual -- GB300 issues float32
//   far faster than float64, so this replaces cuFFT's float64 R2C / C2R;
//   float32 for the float32 operator, replacing cuFFT R2C / C2R and the
//   separate scale pass.
#pragma once

#include "grid.cuh"

namespace mps {

constexpr int kDfMaxStages = 12;

// One axis: N = product of radices (4, 3, 5, 2), Stockham stage s reads
// in[j + r N/R] and writes out[(j / Ns) Ns R + j % Ns + r Ns].
struct DfAxisPlan {
    int N = 0;
    int nst = 0;
    int R[kDfMaxStages];
    int Ns[kDfMaxStages];
    int twoff[kDfMaxStages];   // offset of stage s's twiddles (Ns x R) in the table
    int ntw = 0;
    const float4 *tw = nullptr;  // device table: (cos hi, cos lo, -sin hi, -sin lo) of 2 pi jm r / (Ns R)
};

struct DfPlan3 {
    DfAxisPlan ax[3];
    bool ok = false;
};

// Builds (and caches per device and length) the plans of a grid; ok = false
// when an axis length has a prime factor other than 2, 3, 5, Nx is odd, or an
// axis is longer than 1024.
int df_plan(const GridParams &gp, DfPlan3 *out);

// Forward: double-float real grids ((hi, lo) float pairs, ncomp x [Nz][Ny][Nx]) -> double-float half
// spectra (ncomp x [Nz][Ny][Nx/2+1], float4 per complex value) in spec.
// Inverse: the reverse, unnormalised.  For the dipole operator the z pass of the
// forward transform, the Green's scale and the z pass of the inverse run in one
// kernel (scale_dipole): spec then never holds the unscaled z-transformed data.
int df_forward_xy(const float2 *grid, float4 *spec, int ncomp, const GridParams &gp, const DfPlan3 &pl,
                  cudaStream_t s);
int df_z_scale_dipole(float4 *spec, int nrhs, const GridParams &gp, const DfPlan3 &pl, const double *H,
                      const float2 *tm6, cudaStream_t s);
// The scale tensor of the double-float z pass, 6 double-float entries per
// half-spectrum point (6 x Gc float2), built once per grid.
int df_scale_table(const GridParams &gp, const double *H, float2 *tm6, cudaStream_t s);
int df_inverse_yx(float4 *spec, float2 *grid, int ncomp, const GridParams &gp, const DfPlan3 &pl, cudaStream_t s);

// The same transforms in float32 (float2 per complex value) for the float32
// operator: the z pass, Green's scale and inverse z pass fused as above.
int f32_forward_xy(const float *grid, float2 *spec, int ncomp, const GridParams &gp, const DfPlan3 &pl,
                   cudaStream_t s);
int f32_z_scale_dipole(float2 *spec, int nrhs, const GridParams &gp, const DfPlan3 &pl, const float *H,
                       cudaStream_t s);
int f32_inverse_yx(float2 *spec, float *grid, int ncomp, const GridParams &gp, const DfPlan3 &pl, cudaStream_t s);

}  // namespace mps
