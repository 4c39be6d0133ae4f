// Gradient form of the float32 wave-space operator (inner operator of the
// mixed-precision solve).
//
// The reference operator spreads the three moment components onto three grids
// and scales their spectra by H k k^T / |k|^2.  Since k k^T = (ik)(ik)^*, the same
// operator (up to the sampling error of the Gaussian's derivative) is
//   rho(n) = sum_a m_a . grad_r w_a(n)              one scalar grid per vector
//   phi    = IFFT( H / |k|^2 FFT(rho) )
//   E_a    = h^3 sum_n grad_r w_a(n) phi(n)
// with r = node - x_a and grad_r w = -(4 xi^2 / eta_d) r_d w per axis (separable:
// the per-axis factors w_d and g_d = dw_d/dr_d).  One FFT pair per vector instead
// of three, a third of the grid traffic.  It differs from the reference operator
// by the discretisation error of the derivative (about 1e-5 relative at the
// configurations measured), which the float64-accurate refinement residual
// removes: the mixed solve still converges to the reference operator's solution.
//
// The kernels follow the tiled spread / contract of tiles.cu (one CTA per
// 16 x 16 x TZ tile, deterministic, no atomics).
#include "gradop.cuh"

#include <cstdlib>
#include <cstring>

namespace mps {


// g[a][d][j] = dw_d/dr at stencil node j of axis d (float32).
__global__ void k_grad_factors(const double *__restrict__ x, int64_t n, GridParams gp, const double *__restrict__ w64,
                               float *__restrict__ g32) {
    const int P = gp.P;
    const int lo = (P - 1) / 2;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * 3; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = t / 3;
        const int d = (int)(t % 3);
        const double h = gp.h[d];
        const double xv = x[3 * a + d];
        const double v = __ddiv_rn(xv, h);
        const double af = floor(fabs(v) + 0.5);
        const double node0 = v > 0 ? af : (v < 0 ? -af : 0.0 * af);
        const double base = __dsub_rn(__dmul_rn(node0, h), xv);
        const double c = -4.0 * gp.xi * gp.xi / gp.eta[d];
        for (int j = 0; j < P; ++j) {
            const double r = base + (double)(j - lo) * h;
            g32[(a * 3 + d) * P + j] = (float)(c * r * w64[(a * 3 + d) * P + j]);
        }
    }
}

// H / |k|^2 on the half spectrum (float32), H including 1/G; zero at k = 0.  One
// thread per point of the spectrum's quarter, written to its mirrored points (same
// |k|^2 and H there).
__global__ void k_grad_scale_coef(GridParams gp, const double *__restrict__ H, float *__restrict__ hs) {
    const HalfQuarter q(gp.N);
    const int64_t Gq = q.size();
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Gq; t += (int64_t)gridDim.x * blockDim.x) {
        int ix, iy, iz;
        q.point(t, &ix, &iy, &iz);
        const double kx = fft_freq(ix, gp.N[0]) * gp.kfac[0];
        const double ky = fft_freq(iy, gp.N[1]) * gp.kfac[1];
        const double kz = fft_freq(iz, gp.N[2]) * gp.kfac[2];
        const double k2 = kx * kx + ky * ky + kz * kz;
        const float v = k2 > 0 ? (float)(H[((int64_t)iz * q.Ny + iy) * q.Nxh + ix] / k2) : 0.f;
        mirror_points(q, ix, iy, iz, [&](int64_t i, int, int) { hs[i] = v; });
    }
}

// Owner-computes spread: thread (tx, ty) of the CTA owns the column (X0+tx,
// Y0+ty, Z0..Z0+TZ-1) of the tile and accumulates it in registers over the
// tile's particle list (fixed order: deterministic, no atomics).  Particles are
// staged in chunks with their per-axis factors already aligned to the tile --
// w and dw/dr at every tile column, row and plane, zero where the stencil does
// not reach -- plus masks of the tile columns, rows and planes they cover, so a
// warp (an 8 x 4 patch of the tile's columns: the particle's 10-wide stencil
// often misses one half of the tile in x, which a warp of two full 16-wide rows
// could not skip) skips a particle with one uniform test and otherwise runs a branch-free
// update: value(x,y,z) = (mx gx wy + my wx gy) wz + mz wx wy gz, over the groups
// of 4 tile planes the particle reaches (a plane mask staged with the factors).
// particles staged per barrier interval: 96 measured 0.300 ms per launch at the bench workload against 0.323
// for 32 (fewer barriers, and the warps' uneven shares of a chunk even out), 0.306 for 64 and 0.301 for 128
constexpr int kGChunk = 96;

// Bounds of 5 blocks per SM (48 registers, 36.5 KB of shared memory each): 0.293 ms per launch at the bench
// workload against 0.299 at 4 blocks (64 registers), 0.300 at 6 (spills) and 0.342 unbounded.
// Depth 12 (36 accumulators for 3 vectors, 64 registers) at 4 blocks per SM, depth 16 (48) at 3.
template <int TZ, int NR>
__global__ void __launch_bounds__(256, TZ > 12 ? 3 : (TZ > 8 ? 4 : 5)) k_spread_grad_tiled(const double *__restrict__ m, int64_t n, int r0,
                                                           const int32_t *__restrict__ start,
                                                           const float *__restrict__ w, const float *__restrict__ g,
                                                           GridParams gp, const int64_t *__restrict__ tstart,
                                                           const int32_t *__restrict__ entries, int ntx, int nty,
                                                           float *__restrict__ grid) {
    constexpr int kPos = kTileX + kTileY + TZ;   // aligned positions per particle
    constexpr int kMS = (3 * NR + 3) & ~3;       // moments, padded to a float4 multiple
    __shared__ float2 s_f[kGChunk][kPos];        // (w, dw/dr) at tile columns, rows, planes
    __shared__ __align__(16) float s_m[kGChunk][kMS];
    __shared__ unsigned s_rows[kGChunk];
    __shared__ unsigned s_cols[kGChunk];
    __shared__ unsigned s_planes[kGChunk];
    const int64_t t = blockIdx.x;
    const int bx = (int)(t % ntx), by = (int)((t / ntx) % nty), bz = (int)(t / ((int64_t)ntx * nty));
    const int X0 = bx * kTileX, Y0 = by * kTileY, Z0 = bz * TZ;
    // warp wid owns the 8 x 4 patch (columns 8 (wid & 1) .. +8, rows 4 (wid >> 1) .. +4) of the 16 x 16 tile
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int px = wid & 1, py = wid >> 1;
    const int tx = 8 * px + (lane & 7), ty = 4 * py + (lane >> 3);
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    float acc[TZ][NR];
#pragma unroll
    for (int z = 0; z < TZ; ++z)
#pragma unroll
        for (int r = 0; r < NR; ++r) acc[z][r] = 0.f;
    const int64_t e0 = tstart[t], e1 = tstart[t + 1];
    for (int64_t cb = e0; cb < e1; cb += kGChunk) {
        const int cnt = (int)min((int64_t)kGChunk, e1 - cb);
        if (threadIdx.x < kGChunk) s_rows[threadIdx.x] = s_cols[threadIdx.x] = s_planes[threadIdx.x] = 0u;
        if (threadIdx.x < cnt) {
            const int32_t a = entries[cb + threadIdx.x];
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const double *ma = m + ((int64_t)(r0 + r) * n + a) * 3;
                s_m[threadIdx.x][3 * r + 0] = (float)ma[0];
                s_m[threadIdx.x][3 * r + 1] = (float)ma[1];
                s_m[threadIdx.x][3 * r + 2] = (float)ma[2];
            }
        }
        __syncthreads();
        for (int q = threadIdx.x; q < cnt * kPos; q += blockDim.x) {
            const int pp = q / kPos, k = q - (q / kPos) * kPos;
            const int32_t a = entries[cb + pp];
            const int d = k < kTileX ? 0 : (k < kTileX + kTileY ? 1 : 2);
            const int tpos = k - (d == 0 ? 0 : (d == 1 ? kTileX : kTileX + kTileY));
            const int origin = d == 0 ? X0 : (d == 1 ? Y0 : Z0);
            const int Nd = d == 0 ? Nx : (d == 1 ? Ny : Nz);
            const int node = origin + tpos;
            int j = node - start[3 * (int64_t)a + d];   // stencil index of this tile position
            if (j < 0) j += Nd;
            float2 f = make_float2(0.f, 0.f);
            if (node < Nd && j < P) {
                const int64_t o = (int64_t)a * 3 * P + d * P + j;
                f = make_float2(w[o], g[o]);
                atomicOr(d == 0 ? &s_cols[pp] : (d == 1 ? &s_rows[pp] : &s_planes[pp]), 1u << tpos);
            }
            s_f[pp][k] = f;
        }
        __syncthreads();
        for (int pp = 0; pp < cnt; ++pp) {
            // the particle misses this warp's patch: none of its 4 rows or none of its 8 columns is covered
            if (((s_rows[pp] >> (4 * py)) & 0xFu) == 0u || ((s_cols[pp] >> (8 * px)) & 0xFFu) == 0u) continue;
            const float2 fx = s_f[pp][tx], fy = s_f[pp][kTileX + ty];
            const float gxwy = fx.y * fy.x, wxgy = fx.x * fy.y, wxwy = fx.x * fy.x;
            float cA[NR], cB[NR];
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                cA[r] = s_m[pp][3 * r] * gxwy + s_m[pp][3 * r + 1] * wxgy;
                cB[r] = s_m[pp][3 * r + 2] * wxwy;
            }
            // planes in groups of 4; a group the particle does not reach is skipped (uniform over the CTA)
            const unsigned planes = s_planes[pp];
#pragma unroll
            for (int z0 = 0; z0 < TZ; z0 += 4) {
                if (TZ > 4 && ((planes >> z0) & 0xFu) == 0u) continue;
#pragma unroll
                for (int z = z0; z < z0 + 4 && z < TZ; ++z) {
                    const float2 fz = s_f[pp][kTileX + kTileY + z];
#pragma unroll
                    for (int r = 0; r < NR; ++r) acc[z][r] += cA[r] * fz.x + cB[r] * fz.y;
                }
            }
        }
        __syncthreads();
    }
    const int gxn = X0 + tx, gyn = Y0 + ty;
    if (gxn < Nx && gyn < Ny) {
        const int64_t G = gp.G;
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            const int gz = Z0 + z;
            if (gz < Nz) {
                const int64_t node = ((int64_t)gz * Ny + gyn) * Nx + gxn;
#pragma unroll
                for (int r = 0; r < NR; ++r) grid[(int64_t)(r0 + r) * G + node] = acc[z][r];
            }
        }
    }
}


constexpr int kGRowPad = kTileX + 1;

template <int TZ, int NR>
__global__ void __launch_bounds__(256) k_contract_grad_tiled(const float *__restrict__ grid, int r0,
                                                             const int32_t *__restrict__ start,
                                                             const float *__restrict__ w, const float *__restrict__ g,
                                                             GridParams gp, const int64_t *__restrict__ tstart,
                                                             const int32_t *__restrict__ entries, int ntx, int nty,
                                                             float *__restrict__ partial) {
    constexpr int kPlane = kTileY * kGRowPad;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *tile = (float *)smem_raw;                        // [NR][TZ][16][17]
    float *wbuf = tile + NR * TZ * kPlane;                  // [8 warps][2][3*kMaxP]
    const int64_t t = blockIdx.x;
    const int bx = (int)(t % ntx), by = (int)((t / ntx) % nty), bz = (int)(t / ((int64_t)ntx * nty));
    const int X0 = bx * kTileX, Y0 = by * kTileY, Z0 = bz * TZ;
    const int tx = threadIdx.x & (kTileX - 1), ty = threadIdx.x >> 4;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    const int64_t e0 = tstart[t], e1 = tstart[t + 1];
    if (e0 == e1) return;
    {
        const int gxn = X0 + tx, gyn = Y0 + ty;
        const bool in = gxn < Nx && gyn < Ny;
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            const int gz = Z0 + z;
            const int64_t node = ((int64_t)gz * Ny + gyn) * Nx + gxn;
#pragma unroll
            for (int r = 0; r < NR; ++r)
                tile[(r * TZ + z) * kPlane + ty * kGRowPad + tx] =
                    (in && gz < Nz) ? grid[(int64_t)(r0 + r) * G + node] : 0.f;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float *wb = wbuf + wid * 2 * 3 * kMaxP;
    float *gb = wb + 3 * kMaxP;
    for (int64_t e = e0 + wid; e < e1; e += 8) {
        const int32_t a = entries[e];
        int ox = X0 - start[3 * a], oy = Y0 - start[3 * a + 1], oz = Z0 - start[3 * a + 2];
        if (ox < 0) ox += Nx;
        if (oy < 0) oy += Ny;
        if (oz < 0) oz += Nz;
        for (int k = lane; k < 3 * P; k += 32) {
            wb[(k / P) * kMaxP + (k % P)] = w[(int64_t)a * 3 * P + k];
            gb[(k / P) * kMaxP + (k % P)] = g[(int64_t)a * 3 * P + k];
        }
        int xr = lane - ox, yr = lane - oy, zr = lane - oz;
        if (xr < 0) xr += Nx;
        if (yr < 0) yr += Ny;
        if (zr < 0) zr += Nz;
        const unsigned mx = __ballot_sync(0xffffffffu, lane < P && xr < kTileX && X0 + xr < Nx);
        const unsigned my = __ballot_sync(0xffffffffu, lane < P && yr < kTileY && Y0 + yr < Ny);
        const unsigned mz = __ballot_sync(0xffffffffu, lane < P && zr < TZ && Z0 + zr < Nz);
        __syncwarp();
        const int nx = __popc(mx), ny = __popc(my);
        float acc[3 * NR];
#pragma unroll
        for (int c = 0; c < 3 * NR; ++c) acc[c] = 0.f;
        for (int q = lane; q < nx * ny; q += 32) {
            const int jx = (int)__fns(mx, 0, q % nx + 1), jy = (int)__fns(my, 0, q / nx + 1);
            int xx = jx - ox, yy = jy - oy;
            if (xx < 0) xx += Nx;
            if (yy < 0) yy += Ny;
            float s0[NR], s1[NR];
#pragma unroll
            for (int r = 0; r < NR; ++r) s0[r] = s1[r] = 0.f;
            unsigned mzz = mz;
            while (mzz) {
                const int jz = __ffs(mzz) - 1;
                mzz &= mzz - 1;
                int zz = jz - oz;
                if (zz < 0) zz += Nz;
                const float wz = wb[2 * kMaxP + jz], gz = gb[2 * kMaxP + jz];
                const float *tp = tile + zz * kPlane + yy * kGRowPad + xx;
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    const float v = tp[r * TZ * kPlane];
                    s0[r] += v * wz;
                    s1[r] += v * gz;
                }
            }
            const float wx = wb[jx], wy = wb[kMaxP + jy], gx = gb[jx], gy = gb[kMaxP + jy];
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                acc[3 * r + 0] += gx * wy * s0[r];
                acc[3 * r + 1] += wx * gy * s0[r];
                acc[3 * r + 2] += wx * wy * s1[r];
            }
        }
#pragma unroll
        for (int c = 0; c < 3 * NR; ++c) acc[c] = warp_sum(acc[c]);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 3 * NR; ++c) partial[e * 3 * NR + c] = acc[c];
        }
        __syncwarp();
    }
}

// Each particle's partials summed in its fixed tile order (float64 accumulation).
template <int NR>
__global__ void k_contract_grad_gather(const float *__restrict__ partial, int64_t n, int r0,
                                       const int64_t *__restrict__ pstart, const int32_t *__restrict__ pentry,
                                       double hprod, double *__restrict__ out) {
    constexpr int C = 3 * NR;
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        double acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] = 0.0;
        for (int64_t k = pstart[a]; k < pstart[a + 1]; ++k) {
            const float *pp = partial + (int64_t)pentry[k] * C;
#pragma unroll
            for (int c = 0; c < C; ++c) acc[c] += (double)pp[c];
        }
#pragma unroll
        for (int r = 0; r < NR; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) out[((int64_t)(r0 + r) * n + a) * 3 + c] = acc[3 * r + c] * hprod;
    }
}

// Contraction as a warp-per-particle gather: the grids of the gradient form (one
// per vector) are small enough to be read mostly from L2.  Lanes take the (x, y)
// columns of the stencil, each runs its z column; fixed summation order.  Warps
// visit particles in `order` (spatially sorted: the warps of one CTA read
// overlapping stencils, so much of it comes from L1); null = input order.
// 3 blocks per SM (79 registers for 3 vectors, no spills): 0.283 ms per launch at the bench workload against 0.293
// with the 64-register cap of 4 blocks (which spills) and 0.338 with 2 blocks
template <int NR>
__global__ void __launch_bounds__(256, 3) k_contract_grad_warp(const float *__restrict__ grid, int64_t n, int r0,
                                                            const int32_t *__restrict__ order,
                                                            const int32_t *__restrict__ start,
                                                            const float *__restrict__ w, const float *__restrict__ g,
                                                            GridParams gp, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int P = gp.P;
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    for (int64_t i = warp; i < n; i += nw) {
        const int64_t a = order ? order[i] : i;
        const int sx = start[3 * a], sy = start[3 * a + 1], sz = start[3 * a + 2];
        const float *wa = w + a * 3 * P, *ga = g + a * 3 * P;
        float acc[3 * NR];
#pragma unroll
        for (int c = 0; c < 3 * NR; ++c) acc[c] = 0.f;
        for (int row0 = 0; row0 < P * P; row0 += 32) {
            int idx, sub, lpp;
            if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
            const int jx = idx % P, jy = idx / P;
            int ix = sx + jx;
            if (ix >= Nx) ix -= Nx;
            int iy = sy + jy;
            if (iy >= Ny) iy -= Ny;
            const int64_t rowb = (int64_t)ix + (int64_t)Nx * iy;
            float s0[NR], s1[NR];
#pragma unroll
            for (int r = 0; r < NR; ++r) s0[r] = s1[r] = 0.f;
            // unrolled over the whole z run of P = 10 (10 x NR loads in flight per lane; 5 and 2 measured slower)
#pragma unroll 10
            for (int jz = sub; jz < P; jz += lpp) {
                int iz = sz + jz;
                if (iz >= Nz) iz -= Nz;
                const int64_t node = rowb + (int64_t)Nx * Ny * iz;
                const float wz = wa[2 * P + jz], gz = ga[2 * P + jz];
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    const float v = __ldg(grid + (int64_t)(r0 + r) * G + node);
                    s0[r] += v * wz;
                    s1[r] += v * gz;
                }
            }
            const float wx = wa[jx], wy = wa[P + jy], gx = ga[jx], gy = ga[P + jy];
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                acc[3 * r + 0] += gx * wy * s0[r];
                acc[3 * r + 1] += wx * gy * s0[r];
                acc[3 * r + 2] += wx * wy * s1[r];
            }
        }
#pragma unroll
        for (int c = 0; c < 3 * NR; ++c) acc[c] = warp_sum(acc[c]);
        if (lane == 0)
#pragma unroll
            for (int r = 0; r < NR; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    out[((int64_t)(r0 + r) * n + a) * 3 + c] = (double)acc[3 * r + c] * gp.hprod;
    }
}

// Contraction by home blocks (the default where the support is 8 or 10): one CTA per
// kHomeBlock^3 block of grid nodes stages every node its particles' stencils can
// reach -- the block grown by P - 1 nodes per axis, R = kHomeBlock + P - 1 per axis,
// one plane of R^3 floats per vector -- in shared memory with coalesced loads, and
// its particles' offsets and per-axis factors (kHomeChunk particles at a time).  One
// warp per particle then runs the sums of k_contract_grad_warp in the same order,
// from shared memory and registers instead of L2: the results are bit-identical.  P
// is a template parameter, so the z runs unroll completely with the z factors in
// registers and the shared-memory offsets are immediates.  A node is staged by about
// (R / kHomeBlock)^3 blocks (9.6 at P = 10), all from L2.
// 67 KB of shared memory at P = 10 and 3 vectors, 3 blocks per SM (80 registers): the mixed step at the bench
// workload took 19.25 ms against 20.08 with the warp gather; float4 nodes (the 3 vectors interleaved, 87 KB,
// 2 blocks per SM) took 20.17.
constexpr int kHomeChunk = 32;

template <int NR, int P>
constexpr size_t home_smem_bytes() {
    constexpr int R = kHomeBlock + P - 1;
    return sizeof(float) * (size_t)NR * R * R * R + sizeof(float) * 2 * kHomeChunk * 3 * P +
           sizeof(int) * 4 * kHomeChunk;
}

template <int NR, int P>
__global__ void __launch_bounds__(256, 3) k_contract_grad_home(const float *__restrict__ grid, int64_t n, int r0,
                                                               const int64_t *__restrict__ hstart,
                                                               const int32_t *__restrict__ hentries, int nbx, int nby,
                                                               const int32_t *__restrict__ start,
                                                               const float *__restrict__ w, const float *__restrict__ g,
                                                               GridParams gp, double *__restrict__ out) {
    constexpr int R = kHomeBlock + P - 1;
    constexpr int RR = R * R;
    constexpr int VOL = RR * R;
    constexpr int F = 3 * P;                        // per-axis factors of one particle
    extern __shared__ float s_reg[];                // [NR][VOL] nodes, x fastest
    float *s_w = s_reg + NR * VOL;                  // [kHomeChunk][F]
    float *s_g = s_w + kHomeChunk * F;              // [kHomeChunk][F]
    int *s_p = (int *)(s_g + kHomeChunk * F);       // [kHomeChunk][4]: offsets in the block, particle id
    const int64_t b = blockIdx.x;
    const int64_t e0 = hstart[b], e1 = hstart[b + 1];
    if (e0 == e1) return;   // the whole CTA leaves: no barrier is left waiting
    const int Nx = gp.N[0], Ny = gp.N[1], Nz = gp.N[2];
    const int64_t G = gp.G;
    const int X0 = (int)(b % nbx) * kHomeBlock, Y0 = (int)((b / nbx) % nby) * kHomeBlock,
              Z0 = (int)(b / ((int64_t)nbx * nby)) * kHomeBlock;
    const float *g0 = grid + (int64_t)r0 * G;
#pragma unroll 4
    for (int q = threadIdx.x; q < VOL; q += blockDim.x) {
        const int row = q / R, x = q - row * R;
        const int z = row / R, y = row - z * R;
        // origin + offset < 3 N (the host requires N >= kHomeBlock and N >= P): at most two wraps
        int gx = X0 + x, gy = Y0 + y, gz = Z0 + z;
        gx -= gx >= Nx ? Nx : 0;
        gx -= gx >= Nx ? Nx : 0;
        gy -= gy >= Ny ? Ny : 0;
        gy -= gy >= Ny ? Ny : 0;
        gz -= gz >= Nz ? Nz : 0;
        gz -= gz >= Nz ? Nz : 0;
        const int64_t node = ((int64_t)gz * Ny + gy) * Nx + gx;
#pragma unroll
        for (int r = 0; r < NR; ++r) s_reg[r * VOL + q] = __ldg(g0 + r * G + node);
    }
    const int lane = threadIdx.x & 31;
    for (int64_t c0 = e0; c0 < e1; c0 += kHomeChunk) {
        const int cnt = (int)min((int64_t)kHomeChunk, e1 - c0);
        for (int q = threadIdx.x; q < cnt * F; q += blockDim.x) {
            const int p = q / F, k = q - p * F;
            const int64_t a = hentries[c0 + p];
            s_w[q] = w[a * F + k];
            s_g[q] = g[a * F + k];
        }
        if (threadIdx.x < cnt) {
            const int64_t a = hentries[c0 + threadIdx.x];
            // the home block holds the stencil's first node: offsets in [0, kHomeBlock)
            s_p[4 * threadIdx.x + 0] = start[3 * a] - X0;
            s_p[4 * threadIdx.x + 1] = start[3 * a + 1] - Y0;
            s_p[4 * threadIdx.x + 2] = start[3 * a + 2] - Z0;
            s_p[4 * threadIdx.x + 3] = (int)a;
        }
        __syncthreads();   // the region (first pass) and this chunk's particle data are in place
        for (int pp = threadIdx.x >> 5; pp < cnt; pp += blockDim.x >> 5) {
            const int ox = s_p[4 * pp], oy = s_p[4 * pp + 1], oz = s_p[4 * pp + 2];
            const int64_t a = s_p[4 * pp + 3];
            const float *wa = s_w + pp * F, *ga = s_g + pp * F;
            float wz[P], gz[P];
#pragma unroll
            for (int j = 0; j < P; ++j) {
                wz[j] = wa[2 * P + j];
                gz[j] = ga[2 * P + j];
            }
            float acc[3 * NR];
#pragma unroll
            for (int c = 0; c < 3 * NR; ++c) acc[c] = 0.f;
#pragma unroll
            for (int row0 = 0; row0 < P * P; row0 += 32) {
                int idx, sub, lpp;   // lpp is a constant of each unrolled round
                if (!stencil_row(row0, P, lane, &idx, &sub, &lpp)) continue;
                const int jx = idx % P, jy = idx / P;
                const float *col = s_reg + (oz * R + oy + jy) * R + ox + jx;
                float s0[NR], s1[NR];
#pragma unroll
                for (int r = 0; r < NR; ++r) s0[r] = s1[r] = 0.f;
                if (lpp == 1) {
#pragma unroll
                    for (int jz = 0; jz < P; ++jz) {
#pragma unroll
                        for (int r = 0; r < NR; ++r) {
                            const float v = col[r * VOL + jz * RR];
                            s0[r] += v * wz[jz];
                            s1[r] += v * gz[jz];
                        }
                    }
                } else {
                    for (int jz = sub; jz < P; jz += lpp) {
                        const float wzj = wa[2 * P + jz], gzj = ga[2 * P + jz];
#pragma unroll
                        for (int r = 0; r < NR; ++r) {
                            const float v = col[r * VOL + jz * RR];
                            s0[r] += v * wzj;
                            s1[r] += v * gzj;
                        }
                    }
                }
                const float wx = wa[jx], wy = wa[P + jy], gx = ga[jx], gy = ga[P + jy];
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    acc[3 * r + 0] += gx * wy * s0[r];
                    acc[3 * r + 1] += wx * gy * s0[r];
                    acc[3 * r + 2] += wx * wy * s1[r];
                }
            }
#pragma unroll
            for (int c = 0; c < 3 * NR; ++c) acc[c] = warp_sum(acc[c]);
            if (lane == 0)
#pragma unroll
                for (int r = 0; r < NR; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        out[((int64_t)(r0 + r) * n + a) * 3 + c] = (double)acc[3 * r + c] * gp.hprod;
        }
        __syncthreads();   // this chunk's particle data is read before the next chunk overwrites it
    }
}

bool contract_grad_home_supported(const GridParams &gp) {
    if (gp.P != 8 && gp.P != 10) return false;
    for (int d = 0; d < 3; ++d)
        if (gp.N[d] < kHomeBlock || gp.N[d] < gp.P) return false;
    return true;
}

template <int NR, int P>
static int home_launch(const float *grid, int64_t n, int r0, const int32_t *start, const float *w, const float *g,
                       const GridParams &gp, const TileBins &tb, double *out, cudaStream_t s) {
    constexpr size_t smem = home_smem_bytes<NR, P>();
    if (smem > 48 * 1024)
        MPS_CUDA_TRY(cudaFuncSetAttribute(k_contract_grad_home<NR, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    k_contract_grad_home<NR, P><<<(unsigned)tb.nhome, 256, smem, s>>>(grid, n, r0, tb.hstart, tb.hentries, tb.nhb[0],
                                                                       tb.nhb[1], start, w, g, gp, out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <int P>
static int home_dispatch(const float *grid, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                         const GridParams &gp, const TileBins &tb, double *out, cudaStream_t s) {
    for (int r0 = 0; r0 < nrhs; r0 += 3) {
        const int nr = min(3, nrhs - r0);
        const int rc = nr == 3   ? home_launch<3, P>(grid, n, r0, start, w, g, gp, tb, out, s)
                       : nr == 2 ? home_launch<2, P>(grid, n, r0, start, w, g, gp, tb, out, s)
                                 : home_launch<1, P>(grid, n, r0, start, w, g, gp, tb, out, s);
        if (rc) return rc;
    }
    return MPS_OK;
}

int contract_grad_home(const float *grid, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                       const GridParams &gp, const TileBins &tb, double *out, cudaStream_t s) {
    if (!tb.has_home || !contract_grad_home_supported(gp)) return MPS_BAD_ARG;
    if (gp.P == 10) return home_dispatch<10>(grid, n, nrhs, start, w, g, gp, tb, out, s);
    return home_dispatch<8>(grid, n, nrhs, start, w, g, gp, tb, out, s);
}

int contract_grad_warp(const float *grid, int64_t n, int nrhs, const int32_t *order, const int32_t *start,
                       const float *w, const float *g, const GridParams &gp, double *out, cudaStream_t s) {
    const unsigned blocks = grid_for(n * 32, 256, 152 * 64);
    for (int r0 = 0; r0 < nrhs; r0 += 3) {
        const int nr = min(3, nrhs - r0);
        if (nr == 3)
            k_contract_grad_warp<3><<<blocks, 256, 0, s>>>(grid, n, r0, order, start, w, g, gp, out);
        else if (nr == 2)
            k_contract_grad_warp<2><<<blocks, 256, 0, s>>>(grid, n, r0, order, start, w, g, gp, out);
        else
            k_contract_grad_warp<1><<<blocks, 256, 0, s>>>(grid, n, r0, order, start, w, g, gp, out);
        MPS_LAUNCH_CHECK();
    }
    return MPS_OK;
}

int grad_factors(const double *x, int64_t n, const GridParams &gp, const double *w64, float *g32, cudaStream_t s) {
    k_grad_factors<<<grid_for(3 * n, 256), 256, 0, s>>>(x, n, gp, w64, g32);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

int grad_scale_coef(const GridParams &gp, const double *H, float *hs, cudaStream_t s) {
    k_grad_scale_coef<<<grid_for(HalfQuarter(gp.N).size(), 256), 256, 0, s>>>(gp, H, hs);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <int TZ, int NR>
static int grad_launch(const double *m, int64_t n, int r0, const int32_t *start, const float *w, const float *g,
                       const GridParams &gp, const TileBins &tb, float *grid, float *partial, double *out,
                       bool spread_phase, cudaStream_t s) {
    if (spread_phase) {
        k_spread_grad_tiled<TZ, NR><<<(unsigned)tb.ntiles, 256, 0, s>>>(m, n, r0, start, w, g, gp, tb.tile_start,
                                                                         tb.entries, tb.ntx, tb.nty, grid);
        MPS_LAUNCH_CHECK();
        return MPS_OK;
    }
    const size_t smem = sizeof(float) * ((size_t)NR * TZ * kTileY * kGRowPad + 8 * 2 * 3 * kMaxP);
    if (smem > 48 * 1024)
        MPS_CUDA_TRY(cudaFuncSetAttribute(k_contract_grad_tiled<TZ, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    k_contract_grad_tiled<TZ, NR><<<(unsigned)tb.ntiles, 256, smem, s>>>(grid, r0, start, w, g, gp, tb.tile_start,
                                                                          tb.entries, tb.ntx, tb.nty, partial);
    MPS_LAUNCH_CHECK();
    k_contract_grad_gather<NR><<<grid_for(n, 256), 256, 0, s>>>(partial, n, r0, tb.pstart, tb.pentry, gp.hprod, out);
    MPS_LAUNCH_CHECK();
    return MPS_OK;
}

template <int TZ>
static int grad_dispatch(const double *m, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                         const GridParams &gp, const TileBins &tb, float *grid, float *partial, double *out,
                         bool spread_phase, cudaStream_t s) {
    for (int r0 = 0; r0 < nrhs; r0 += 3) {
        const int nr = min(3, nrhs - r0);
        int rc = nr == 3   ? grad_launch<TZ, 3>(m, n, r0, start, w, g, gp, tb, grid, partial, out, spread_phase, s)
                 : nr == 2 ? grad_launch<TZ, 2>(m, n, r0, start, w, g, gp, tb, grid, partial, out, spread_phase, s)
                           : grad_launch<TZ, 1>(m, n, r0, start, w, g, gp, tb, grid, partial, out, spread_phase, s);
        if (rc) return rc;
    }
    return MPS_OK;
}

template <int TZ>
static int spread_grad_deep(const double *m, int64_t n, int nrhs, const int32_t *start, const float *w,
                            const float *g, const GridParams &gp, const TileBins &tb, float *grid, cudaStream_t s) {
    for (int r0 = 0; r0 < nrhs; r0 += 3) {
        const int nr = min(3, nrhs - r0);
        const unsigned blocks = (unsigned)tb.ntiles;
        if (nr == 3)
            k_spread_grad_tiled<TZ, 3><<<blocks, 256, 0, s>>>(m, n, r0, start, w, g, gp, tb.tile_start, tb.entries,
                                                              tb.ntx, tb.nty, grid);
        else if (nr == 2)
            k_spread_grad_tiled<TZ, 2><<<blocks, 256, 0, s>>>(m, n, r0, start, w, g, gp, tb.tile_start, tb.entries,
                                                              tb.ntx, tb.nty, grid);
        else
            k_spread_grad_tiled<TZ, 1><<<blocks, 256, 0, s>>>(m, n, r0, start, w, g, gp, tb.tile_start, tb.entries,
                                                              tb.ntx, tb.nty, grid);
        MPS_LAUNCH_CHECK();
    }
    return MPS_OK;
}

int spread_grad_tiled(const double *m, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                      const GridParams &gp, const TileBins &tb, float *grid, cudaStream_t s) {
    if (tb.tz == 16) return spread_grad_deep<16>(m, n, nrhs, start, w, g, gp, tb, grid, s);
    if (tb.tz == 12) return spread_grad_deep<12>(m, n, nrhs, start, w, g, gp, tb, grid, s);
    if (tb.tz == 8) return grad_dispatch<8>(m, n, nrhs, start, w, g, gp, tb, grid, nullptr, nullptr, true, s);
    if (tb.tz == 4) return grad_dispatch<4>(m, n, nrhs, start, w, g, gp, tb, grid, nullptr, nullptr, true, s);
    return MPS_BAD_ARG;
}

int contract_grad_tiled(const float *grid, int64_t n, int nrhs, const int32_t *start, const float *w, const float *g,
                        const GridParams &gp, const TileBins &tb, float *partial, double *out, cudaStream_t s) {
    float *gr = const_cast<float *>(grid);
    if (tb.tz == 8) return grad_dispatch<8>(nullptr, n, nrhs, start, w, g, gp, tb, gr, partial, out, false, s);
    if (tb.tz == 4) return grad_dispatch<4>(nullptr, n, nrhs, start, w, g, gp, tb, gr, partial, out, false, s);
    return MPS_BAD_ARG;
}

}  // namespace mps
