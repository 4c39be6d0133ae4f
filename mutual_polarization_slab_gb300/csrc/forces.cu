// Point-dipole pair forces and energies for fixed dipoles
// (CPU - HOOMD simulation test/dipole_forces_ext/_dipole_forces_ext.cpp:119-452).
//
// One thread per particle gathers over the 27 surrounding cells (cell edge >=
// r_cut, at least 3 cells per axis): every pair is evaluated from both ends, so
// forces and energies need no atomics and the summation order is fixed.  The
// pair terms are the reference's: minimum image d - L rint(d/L) (z only when
// periodic), 1e-24 <= r^2 <= r_cut^2,
//   U = pref [(mi.mj)/r^3 - 3 (mi.r)(mj.r)/r^5], half to each particle,
//   F_i = 3 pref / r^5 [(mi.mj) r + (mj.r) mi + (mi.r) mj - 5 (mi.r)(mj.r) r / r^2].
#include "cells.cuh"

namespace mps {

__global__ void k_dipole_forces(const double *__restrict__ pos, const double *__restrict__ dip, int64_t n,
                                double Lx, double Ly, double Lz, int periodic_z, double rc2, double pref,
                                const int32_t *__restrict__ lin, const int32_t *__restrict__ counts,
                                const int64_t *__restrict__ starts, const int32_t *__restrict__ sorted, int64_t ncx,
                                int64_t ncy, int64_t ncz, double *__restrict__ F, double *__restrict__ pe) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
        const double mxi = dip[3 * i], myi = dip[3 * i + 1], mzi = dip[3 * i + 2];
        const int32_t c = lin[i];
        const int64_t cx = c % ncx, cy = (c / ncx) % ncy, cz = c / (ncx * ncy);
        double fx = 0.0, fy = 0.0, fz = 0.0, e = 0.0;
        for (int o = 0; o < 27; ++o) {
            const int64_t nx = wrap_index(cx + (o / 9) - 1, ncx);
            const int64_t ny = wrap_index(cy + (o / 3) % 3 - 1, ncy);
            const int64_t nz = wrap_index(cz + o % 3 - 1, ncz);
            const int64_t nb = nx + ncx * (ny + ncy * nz);
            const int64_t b0 = starts[nb], len = counts[nb];
            for (int64_t q = 0; q < len; ++q) {
                const int32_t j = sorted[b0 + q];
                if (j == i) continue;
                double dx = xi - pos[3 * j], dy = yi - pos[3 * j + 1], dz = zi - pos[3 * j + 2];
                dx -= Lx * rint(dx / Lx);
                dy -= Ly * rint(dy / Ly);
                if (periodic_z) dz -= Lz * rint(dz / Lz);
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > rc2 || r2 < 1e-24) continue;
                const double inv_r2 = 1.0 / r2;
                const double inv_r = sqrt(inv_r2);
                const double inv_r3 = inv_r2 * inv_r;
                const double inv_r5 = inv_r3 * inv_r2;
                const double mxj = dip[3 * j], myj = dip[3 * j + 1], mzj = dip[3 * j + 2];
                const double mimj = mxi * mxj + myi * myj + mzi * mzj;
                const double mir = mxi * dx + myi * dy + mzi * dz;
                const double mjr = mxj * dx + myj * dy + mzj * dz;
                const double U = pref * (mimj * inv_r3 - 3.0 * (mir * mjr) * inv_r5);
                const double coef = pref * 3.0 * inv_r5;
                const double s5 = 5.0 * (mir * mjr) * inv_r2;
                fx += coef * (mimj * dx + mjr * mxi + mir * mxj - s5 * dx);
                fy += coef * (mimj * dy + mjr * myi + mir * myj - s5 * dy);
                fz += coef * (mimj * dz + mjr * mzi + mir * mzj - s5 * dz);
                e += 0.5 * U;
            }
        }
        F[3 * i] = fx;
        F[3 * i + 1] = fy;
        F[3 * i + 2] = fz;
        pe[i] = e;
    }
}

}  // namespace mps

using namespace mps;

extern "C" int mps_dipole_forces(const double *pos, const double *dip, int64_t n, const double *box, double r_cut,
                                 double prefactor, int32_t periodic_z, double *forces, double *pe,
                                 mps_stream_t stream) {
    if (n < 0 || !box || (n > 0 && (!pos || !dip || !forces || !pe))) return MPS_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (!(box[d] > 0)) return MPS_BAD_ARG;
    if (!(r_cut > 0)) return MPS_BAD_ARG;
    if (r_cut >= 0.5 * fmin(box[0], box[1])) return MPS_RC_GT_HALF_BOX;
    if (periodic_z && r_cut >= 0.5 * box[2]) return MPS_RC_GT_HALF_BOX;
    if (n == 0) return MPS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int64_t ncell[3];
    compute_ncell(box, r_cut, ncell);
    const int64_t ncells = ncell[0] * ncell[1] * ncell[2];
    int64_t *cell3 = nullptr;
    void *bins = nullptr;
    MPS_CUDA_TRY(cudaMallocAsync((void **)&cell3, sizeof(int64_t) * 3 * n, s));
    MPS_CUDA_TRY(cudaMallocAsync(&bins, cell_bins_bytes(n, ncells), s));
    CellBins cb;
    int rc = cell_assign(pos, n, box, ncell, cell3, s);
    if (!rc) rc = cell_bins_build(cell3, n, ncell, bins, cb, s);
    if (!rc) {
        k_dipole_forces<<<grid_for(n, 128), 128, 0, s>>>(pos, dip, n, box[0], box[1], box[2], periodic_z,
                                                         r_cut * r_cut, prefactor, cb.lin, cb.counts, cb.starts,
                                                         cb.sorted, ncell[0], ncell[1], ncell[2], forces, pe);
        count_launch();
        if (cudaGetLastError() != cudaSuccess) rc = MPS_CUDA_ERR;
    }
    cudaFreeAsync(cell3, s);
    cudaFreeAsync(bins, s);
    return rc;
}
