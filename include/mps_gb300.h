/*
 * mps_gb300.h -- C ABI of the GB300 spectral-Ewald mutual-polarisation solve.
 *
 * Every entry point takes caller-owned DEVICE pointers (unless marked "host"),
 * plain sizes, and the CUDA stream to run on; it returns an int status
 * (enum mps_status).  No C++ exception crosses this boundary and no entry
 * point synchronises the device except where an output size is data
 * dependent (the *_count calls) or a Krylov solve reads its convergence flags.
 *
 * Array layouts (all row-major / C order, element type as declared):
 *   positions   x[n][3]            float64
 *   moments     m[nvec][n][3]      float64  (nvec independent real vectors;
 *                                            the Python layer passes the real
 *                                            and imaginary parts of a complex
 *                                            array as nvec = 2)
 *   grids       g[nvec][3][Nz][Ny][Nx] float64, x fastest -- the same linear
 *                                            node index ix + Nx*iy + Nx*Ny*iz as
 *                                            the reference's Fortran-ordered grids
 *   pair lists  int64, directed, p1[k] receives the field of p2[k]
 *
 * Reference interfaces are cited as EW/<file>:<lines> for
 * "CPU - Ewald test/<file>" and CH/<file> for "Capacitance_Hetero/<file>".
 */
#ifndef MPS_GB300_H
#define MPS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t (a CUstream). NULL = the legacy default stream. */
typedef struct CUstream_st *mps_stream_t;

enum mps_status {
    MPS_OK = 0,
    MPS_BAD_ARG = 1,          /* ValueError in the reference's Python layer        */
    MPS_RC_GT_HALF_BOX = 2,   /* EW/capacitance.py:364-365                         */
    MPS_TABLE_RANGE = 3,      /* EW/ewald.py:999-1007 separation outside the table */
    MPS_NOT_CONVERGED = 4,    /* GMRES hit maxit (the reference ignores its flag)   */
    MPS_CUDA_ERR = 5,
    MPS_CUFFT_ERR = 6,
    MPS_NO_MEMORY = 7,
    MPS_SCRATCH_LIMIT = 8     /* input or output larger than a fixed-size buffer  */
};

enum mps_precision {
    MPS_FP64 = 0,             /* every stage in float64                              */
    MPS_FP32 = 1,             /* float32 matvec (grids, FFT, pair sum), float64 I/O  */
    MPS_FP32_GRAD = 3,        /* float32 matvec in gradient form: the moments spread */
                              /* as one scalar grid sum m.grad w per vector, scaled  */
                              /* by H/|k|^2, contracted with grad w (one FFT pair per */
                              /* vector instead of three; differs from the reference */
                              /* operator by the derivative's sampling error, about  */
                              /* 1e-5 relative; dipole operator with tiled kernels,  */
                              /* else MPS_FP32)                                       */
    MPS_DF = 2                /* float64 matvec whose FFTs and Green's scale run in  */
                              /* double-float arithmetic (float hi + float lo,       */
                              /* ~48-bit significand; dipole operator, grid axes of  */
                              /* factors 2, 3, 5 up to 1024, even Nx; otherwise the  */
                              /* float64 path)                                        */
};

const char *mps_status_string(int status);
/* 5: adds mps_batch_item and mps_solve_batched (4: the inner-grid fields of mps_system_desc). */
int mps_abi_version(void);

/* ------------------------------------------------------------------------- */
/* Stateless operators (the reference's ewald.py functions, one each)         */
/* ------------------------------------------------------------------------- */

/* Replaces EW/ewald.py:604-931 real_space_table(r, xi).
 * r: n separations (no zero).  tables: 6 x (n+1) float64, rows pot_charge,
 * pot_dip, field_dip_1, field_dip_2, field_dip_force_1, field_dip_force_2,
 * each with its r = 0 self value in column 0. */
int mps_real_space_table(const double *r, int64_t n, double xi, double *tables, mps_stream_t stream);

/* Replaces Compute_Field/RealSpaceTable.m:1-150 (the tables of the probe-point field map):
 * as mps_real_space_table, with field_dip_1 and field_dip_2 free of the r < 2
 * overlap polynomial (Compute_Field/RealSpaceTable.m:80-86, 102-109 comment it out). */
int mps_real_space_table_probe(const double *r, int64_t n, double xi, double *tables, mps_stream_t stream);

/* Replaces Compute_Field/FieldMap.m:1-59 with its MagneticField.m:1-74 and
 * RealSpace.m:1-60 (and the probe/particle neighbour list of NeighborList_Types.m):
 * the field at n_e probe points x_e (n_e x 3) from n_p dipoles p (n_p x 3) at x_p,
 * E = -(wave-space part contracted at the probes + real-space part), as FieldMap
 * returns it.  Ngrid, P, eta[3], rc as the caller derives them (FieldMap.m:24-33);
 * perp / para / rvals: field_dip_1 / field_dip_2 of mps_real_space_table_probe and
 * their separations (rvals[0] = 0), n_tab rows.  Real-space pairs with d >= rc or
 * d = 0 are skipped (RealSpace.m:33).  with_real = 0 leaves the real-space part
 * out (a caller with its own probe/particle pair list, FieldMap.m:44-45, adds it).  All pointers are float64 device arrays except
 * box, Ngrid and eta (host).  MPS_RC_GT_HALF_BOX when rc > L/2 on an axis
 * (FieldMap.m:36-39); MPS_TABLE_RANGE when a separation is beyond the table. */
int mps_field_map(const double *x_e, int64_t n_e, const double *x_p, const double *p, int64_t n_p,
                  const double *box, double xi, double rc, const int64_t *Ngrid, int32_t P, const double *eta,
                  const double *perp, const double *para, const double *rvals, int64_t n_tab, int32_t with_real,
                  double *E, mps_stream_t stream);

/* Replaces Compute_Field_Quadrupole/RealSpaceTable.m (the tables of the quadrupole field map):
 * as mps_quad_table, without the r < 2 overlap polynomials (that file comments them all out). */
int mps_quad_table_probe(const double *r, int64_t n, double xi, double *tables, mps_stream_t stream);

/* Replaces Compute_Field_Quadrupole/FieldMap.m:1-58 with its MatrixVectorMultiply.m:1-80 and
 * RealSpace.m:1-77: field E and field gradient G at n_e probe points x_e from dipoles and
 * quadrupoles sq (n_p x 8: S x y z, Q xx xy xz yy yz) at x_p.  EG: n_e x 8 (E then G), both with
 * FieldMap's sign (-(wave + real)).  tab9: 9 x n_tab device tables on rvals in the order
 * field_dip_1, field_dip_2, field_quad_1..3, grad_quad_1..4 (mps_real_space_table_probe rows 2-3 and
 * mps_quad_table_probe).  Other arguments and status codes as mps_field_map; a source exactly at a
 * probe (d = 0, where the reference divides by zero) is skipped. */
int mps_field_map_quad(const double *x_e, int64_t n_e, const double *x_p, const double *sq, int64_t n_p,
                       const double *box, double xi, double rc, const int64_t *Ngrid, int32_t P, const double *eta,
                       const double *tab9, const double *rvals, int64_t n_tab, int32_t with_real, double *EG,
                       mps_stream_t stream);

/* Replaces Compute_Field_Sizes/FieldMap.m:1-43 with its ComputeField.m:1-40 and RealSpace.m:1-77:
 * field at n_e probe points from dipoles p of n_p spheres of radii `radius` (classes radius_class
 * among n_class distinct radii); the probes are spheres of the smallest radius (ComputeField.m:33).
 * eta: the scalar spectral splitting; perp / para: the M(M+1)/2 table columns (Ep_perp, Ep_para of
 * mps_sizes_table, n_tab rows each) on rvals (FieldMap.m uses 0.5 .. rc + 0.01; separations below
 * rvals[0] or above rvals[n_tab-1] return MPS_TABLE_RANGE).  E = -(wave + real), FieldMap's sign. */
int mps_field_map_sizes(const double *x_e, int64_t n_e, const double *x_p, const double *radius,
                        const int32_t *radius_class, int32_t n_class, const double *p, int64_t n_p,
                        const double *box, double xi, double rc, const int64_t *Ngrid, int32_t P, double eta,
                        const double *perp, const double *para, const double *rvals, int64_t n_tab,
                        int32_t with_real, double *E, mps_stream_t stream);

/* Replaces the dipole + quadrupole couplings of Capacitance_Quadrupole/RealSpaceTable.m:171-378.
 * r: n separations (no zero).  tables: 7 x (n+1) float64, rows field_quad_1,
 * field_quad_2, field_quad_3, grad_quad_1, grad_quad_2, grad_quad_3, grad_quad_4,
 * each with its r = 0 value in column 0 (the grad_quad_2 self value, zero for
 * the others).  field_dip_1/2 come from mps_real_space_table. */
int mps_quad_table(const double *r, int64_t n, double xi, double *tables, mps_stream_t stream);

/* Replaces Capacitance_Sizes/RealSpaceTable.m:1-149 [Ep_perp, Ep_para] = RealSpaceTable(r, a, xi).
 * r: device n separations with r[0] = 0 (row 0 holds the r -> 0 value).
 * a_uniq: device M distinct radii.  perp, para: device M(M+1)/2 x n, column of
 * radii pair (i <= j) at index i M - i (i - 1) / 2 + (j - i), each column contiguous. */
int mps_sizes_table(const double *r, int64_t n, const double *a_uniq, int64_t M, double xi, double *perp,
                    double *para, mps_stream_t stream);

/* Replaces EW/ewald.py:84-111 cell_list(x, box, rmax).
 * box: host double[3].  cell: n x 3 int64.  ncell: host int64[3] (output). */
int mps_cell_list(const double *x, int64_t n, const double *box, double rmax,
                  int64_t *cell, int64_t *ncell, mps_stream_t stream);

/* Replaces EW/ewald.py:114-199 neighbor_list(cell, Ncell): two calls sharing a
 * workspace of mps_neighbor_list_workspace() bytes.  _count writes the number of
 * directed candidate pairs to the host int64 *n_pairs (synchronises); _fill
 * writes them in the reference's order into p1, p2 (int64, n_pairs each). */
size_t mps_neighbor_list_workspace(int64_t n, const int64_t *ncell);
int mps_neighbor_list_count(const int64_t *cell, int64_t n, const int64_t *ncell,
                            void *workspace, size_t workspace_bytes, int64_t *n_pairs, mps_stream_t stream);
int mps_neighbor_list_fill(const int64_t *cell, int64_t n, const int64_t *ncell,
                           void *workspace, size_t workspace_bytes, int64_t *p1, int64_t *p2, mps_stream_t stream);

/* Replaces EW/ewald.py:939-1016 prepare_real_space_pairs(x, box, p1, p2, rc, perp, para, rvals).
 * _count keeps the candidates with minimum-image distance d < rc and writes their
 * number to host *n_kept (synchronises); _fill writes p1f, p2f (int64), rhat
 * (n_kept x 3), A, B (float64) in candidate order.  A separation outside
 * rvals returns MPS_TABLE_RANGE. */
size_t mps_real_space_pairs_workspace(int64_t n_cand);
int mps_real_space_pairs_count(const double *x, int64_t n, const double *box, const int64_t *p1,
                               const int64_t *p2, int64_t n_cand, double rc, void *workspace,
                               size_t workspace_bytes, int64_t *n_kept, mps_stream_t stream);
int mps_real_space_pairs_fill(const double *x, int64_t n, const double *box, const int64_t *p1,
                              const int64_t *p2, int64_t n_cand, double rc, const double *perp,
                              const double *para, const double *rvals, int64_t n_tab, void *workspace,
                              size_t workspace_bytes, int64_t *p1f, int64_t *p2f, double *rhat, double *A,
                              double *B, mps_stream_t stream);

/* Replaces EW/ewald.py:1019-1072 real_space_fast(m, lambdap, p1, p2, rhat, A, B, self_perp).
 * m, out: nvec x n x 3.  lambdap: n (the particle permittivity). */
int mps_real_space_fast(const double *m, int64_t n, int64_t nvec, const double *lambdap, const int64_t *p1,
                        const int64_t *p2, const double *rhat, const double *A, const double *B,
                        int64_t n_pairs, double self_perp, double *out, mps_stream_t stream);

/* Replaces EW/ewald.py:205-223 pre_calculations(P, h).  h: host double[3].
 * offset: P^3 x 3 int64, offsetxyz: P^3 x 3 float64. */
int mps_pre_calculations(int P, const double *h, int64_t *offset, double *offsetxyz, mps_stream_t stream);

/* Replaces EW/ewald.py:233-296 prepare_grid_kernel(x, Ngrid, h, xi, eta, P, ...).
 * Ngrid, h, eta: host arrays of 3.  linnode: n x P^3 int64, w_spread and
 * w_contract: n x P^3 float64. */
int mps_grid_kernel(const double *x, int64_t n, const int64_t *Ngrid, const double *h, double xi,
                    const double *eta, int P, int64_t *linnode, double *w_spread, double *w_contract,
                    mps_stream_t stream);

/* Replaces EW/ewald.py:299-331 spread_fast(m, Ngrid, linnode, w_spread).
 * grid: nvec x 3 x G, zeroed by the call. */
int mps_spread_fast(const double *m, int64_t n, int64_t nvec, const int64_t *Ngrid, const int64_t *linnode,
                    const double *w_spread, int64_t P3, double *grid, mps_stream_t stream);

/* Replaces EW/ewald.py:334-368 contract_fast(Htilde, Ngrid, linnode, w_contract).
 * grid: nvec x 3 x G; out: nvec x n x 3. */
int mps_contract_fast(const double *grid, int64_t n, int64_t nvec, const int64_t *Ngrid, const int64_t *linnode,
                      const double *w_contract, int64_t P3, double *out, mps_stream_t stream);

/* Replaces EW/ewald.py:523-582 precompute_kspace(Ngrid, box, xi, eta).
 * khat: Nx x Ny x Nz x 3 float64 (real; the reference stores it as complex with
 * zero imaginary part), Hcoef: Nx x Ny x Nz, both in the reference's fftshift
 * order and C layout. */
int mps_precompute_kspace(const int64_t *Ngrid, const double *box, double xi, const double *eta,
                          double *khat, double *Hcoef, mps_stream_t stream);

/* Replaces EW/ewald.py:585-599 scale_fast(fH, khat, Hcoef).
 * fH, out: interleaved complex128 arrays Nx x Ny x Nz x 3 (C layout). */
int mps_scale_fast(const double *fH, const double *khat, const double *Hcoef, int64_t G, double *out,
                   mps_stream_t stream);

/* ------------------------------------------------------------------------- */
/* System object: everything that depends on positions only, built once per   */
/* solve (the real_precomp / grid_precomp / k_precomp tuples of               */
/* EW/capacitance.py:370-385), plus cuFFT plans and grids.                     */
/* ------------------------------------------------------------------------- */
typedef struct mps_system mps_system;

typedef struct mps_system_desc {
    int64_t n;                /* particles                                         */
    const double *x;          /* device n x 3                                       */
    const double *lambdap;    /* device n_diag x n particle permittivities (eps)   */
    int64_t n_diag;           /* >= 1 permittivity sets (contrast spectrum axis)   */
    double box[3];
    double xi;                /* Ewald splitting parameter                          */
    double rc;                /* real-space cutoff                                  */
    int64_t Ngrid[3];         /* grid nodes per axis                                */
    int32_t P;                /* Gaussian support (nodes per axis)                  */
    double eta[3];            /* spectral splitting; <= 0 derives P (h xi)^2 / pi   */
    const double *perp;       /* device table, field_dip_1 (I - rr part)            */
    const double *para;       /* device table, field_dip_2 (rr part)                */
    const double *rvals;      /* device table separations (rvals[0] = 0)            */
    int64_t n_tab;
    double slab_factor;       /* EW/ewald.py:1233-1236 (1.0 in the reference)       */
    int32_t max_rhs;          /* largest batch of vectors one matvec will take      */
    int32_t kind;             /* MPS_DIPOLE (3 unknowns per sphere),                */
                              /* MPS_DIPOLE_QUADRUPOLE (8: S then Q xx xy xz yy yz) */
                              /* or MPS_POLYDISPERSE (3, spheres of radii a_i)      */
    const double *quad_tables; /* kind MPS_DIPOLE_QUADRUPOLE: device 7 x n_tab on   */
                              /* rvals: field_quad_1..3, grad_quad_1..4, r = 0 first */
                              /* (CQ/RealSpaceTable.m:171-378)                       */
    /* kind MPS_POLYDISPERSE (CS/ComputeField.m:23-57).  perp/para are unused; eta */
    /* is the scalar P (mean(h) xi)^2 / pi in all three entries.                 */
    const double *radius;     /* device n radii                                     */
    const int32_t *radius_class; /* device n class of each radius (0..n_class-1), */
                              /* or NULL: couplings in closed form per pair         */
    int32_t n_class;          /* distinct radii M                                   */
    const double *sizes_tables; /* device 2 x M(M+1)/2 x n_tab: Ep_perp columns then */
                              /* Ep_para columns on rvals (rvals[0] = 0, self first) */
    /* Complex permittivities (kind MPS_DIPOLE; the spectra of CH/CapacitanceSpectrum.m:38-59 and
     * CH/CapacitanceTensorSpectrum.m:38-62 with frequency-dependent eps): device n_diag x n imaginary
     * parts of eps (lambdap holds the real parts), or NULL.  Then every vector of mps_matvec / mps_gmres
     * is complex, stored as 6 float64 per particle (Re m_x, Re m_y, Re m_z, Im m_x, Im m_y, Im m_z),
     * and max_rhs counts complex vectors.  mps_matvec_complex and mps_adjoint_forces are not available. */
    const double *lambdap_imag;
    /* Inner discretisation of the float32 gradient-form operator (MPS_FP32_GRAD, the mixed solve's inner      */
    /* operator; kind MPS_DIPOLE): inner_P > 0 gives it its own grid inner_Ngrid and support inner_P (spectral */
    /* splitting P (h xi)^2 / pi of that grid, the same xi and pair sum).  A coarser grid makes every inner    */
    /* matvec cheaper; the refinement residuals still use the system's own grid, so the mixed solve converges  */
    /* to the same solution.  inner_P = 0: the system's grid.  No counterpart in the reference.                */
    int64_t inner_Ngrid[3];
    int32_t inner_P;
} mps_system_desc;

enum mps_operator_kind { MPS_DIPOLE = 0, MPS_DIPOLE_QUADRUPOLE = 1, MPS_POLYDISPERSE = 2 };

/* Builds cell list, filtered CSR pair list with interpolated couplings, grid
 * geometry, Green's coefficients and FFT plans (EW/capacitance.py:369-385).
 * Allocates device memory; synchronises on the positions' range and the pair
 * count.  A pair separation outside the real-space table is MPS_TABLE_RANGE:
 * returned here for kinds MPS_DIPOLE_QUADRUPOLE and MPS_POLYDISPERSE; for
 * MPS_DIPOLE the check completes on the stream after this call returns (the
 * GPU is still filling the pair list) and the first mps_matvec,
 * mps_matvec_complex, mps_adjoint_forces or mps_gmres call (and every later
 * one) returns it instead. */
int mps_system_create(const mps_system_desc *desc, mps_system **out, mps_stream_t stream);
void mps_system_destroy(mps_system *sys);

/* n_pairs kept (d < rc), cell counts per axis. Host outputs. */
int mps_system_info(const mps_system *sys, int64_t *n_pairs, int64_t *ncell);

/* Replaces EW/ewald.py:1146-1236 magnetic_field for nrhs real vectors.
 * m, out: nrhs x n x 3 float64.  diag_index: host int32[nrhs] selecting the
 * permittivity set of each vector (NULL = set 0).  precision: enum mps_precision.
 * The wave-space part is the real part of the reference's complex pipeline
 * (real-to-complex FFTs; the unpaired Nyquist bins of even axes are coupled
 * symmetrically). */
int mps_matvec(mps_system *sys, const double *m, double *out, int32_t nrhs, const int32_t *diag_index,
               int32_t precision, mps_stream_t stream);

/* Replaces EW/ewald.py:1146-1236 magnetic_field with the reference's complex
 * FFT pipeline, for one complex vector given as m_ri = [Re m; Im m]
 * (2 x n x 3), out_ri the same. */
int mps_matvec_complex(mps_system *sys, const double *m_ri, double *out_ri, int32_t diag_index,
                       mps_stream_t stream);

typedef struct mps_solve_opts {
    double tol;               /* relative residual target ||b - A x|| / ||b||        */
    int32_t restart;          /* inner GMRES steps per cycle                          */
    int32_t maxit;            /* restart cycles (fp64) / refinement steps (mixed)     */
    int32_t precision;        /* MPS_FP64: GMRES on the fp64 operator.
                                 MPS_FP32: iterative refinement, fp64 residuals,
                                 inner GMRES on the fp32 operator                    */
    double inner_tol;         /* mixed: relative tolerance of each inner solve        */
    int32_t inner_maxit;      /* mixed: restart cycles of each inner solve            */
    int32_t residual_policy;  /* mixed: 0 = one float64 residual, later residuals from
                                 the inner GMRES's Arnoldi relation; 1 = a float64
                                 residual after every correction                     */
    int32_t verify;           /* mixed: != 0 ends with a float64 true residual        */
    int32_t residual_precision; /* mixed: operator of the refinement residuals,       */
                              /* MPS_FP64 (0, default) or MPS_DF                      */
    int32_t inner_operator;   /* mixed: operator of the inner GMRES: 0 = float32 of  */
                              /* the reference discretisation, 1 = MPS_FP32_GRAD     */
} mps_solve_opts;

typedef struct mps_solve_info {
    int32_t converged;        /* 1 if relres <= tol                                   */
    int32_t matvecs_fp64;
    int32_t matvecs_fp32;
    int32_t cycles;           /* restart cycles (fp64) or refinement steps (mixed)   */
    double relres;            /* final true relative residual (fp64 operator)        */
} mps_solve_info;

/* Replaces EW/capacitance.py:205-321 magnetic_dipole (GMRES on A m = b) for
 * nrhs right-hand sides solved together (batched matvecs, independent Krylov
 * spaces).  b, x0, x: nrhs x n x 3 float64; x0 may alias x or be NULL (zero).
 * info: host array of nrhs.  Returns MPS_NOT_CONVERGED if any system missed tol. */
int mps_gmres(mps_system *sys, const double *b, const double *x0, double *x, int32_t nrhs,
              const int32_t *diag_index, const mps_solve_opts *opts, mps_solve_info *info,
              mps_stream_t stream);

/* One configuration of a many-configuration solve (mps_solve_batched). */
typedef struct mps_batch_item {
    mps_system_desc desc;       /* the configuration, as for mps_system_create     */
    const double *b;            /* device nrhs x n x ndof right-hand sides          */
    const double *x0;           /* device nrhs x n x ndof guesses, or NULL (zero)   */
    double *x;                  /* device nrhs x n x ndof solutions (not aliasing b) */
    int32_t nrhs;               /* 1 .. desc.max_rhs                                */
    const int32_t *diag_index;  /* host int32[nrhs]: permittivity set of each       */
                                /* right-hand side, or NULL (set 0)                 */
    mps_solve_info *info;       /* host nrhs results, or NULL                       */
    int32_t status;             /* out: this configuration's status                 */
} mps_batch_item;

/* Replaces the loop over configurations of the spectrum drivers (the parfor of
 * CH/CapacitanceTensorSpectrum.m:45 and CS/CapacitanceTensorSpectrum.m:44, each
 * iteration a CapacitanceTensor call): every item is built (mps_system_create),
 * solved (mps_gmres with opts) and released, n_streams configurations at a time,
 * each worker on a host thread and CUDA stream of its own, largest (n x nrhs)
 * first.  The work is ordered after what `stream` holds at the call (the
 * inputs); the call returns once every solution has been written (the host
 * waits, so the call does not belong inside a stream capture).  Each item
 * gets its own status.  Returns MPS_OK when all are MPS_OK, otherwise the
 * status of the first item (in array order) that failed with an error, else
 * MPS_NOT_CONVERGED.  n_streams is capped at 32.  Bad arguments (invalid
 * opts included) return MPS_BAD_ARG before any CUDA work. */
int mps_solve_batched(mps_batch_item *items, int32_t n_items, const mps_solve_opts *opts, int32_t n_streams,
                      mps_stream_t stream);

/* ------------------------------------------------------------------------- */
/* Adjoint forces (no counterpart in the reference, which computes forces from */
/* fixed point dipoles only)                                                   */
/* ------------------------------------------------------------------------- */

/* Forces F = -dE/dx of E = -1/2 m.H0 for the converged moments m (n x 3, one
 * field) of a dipole system, using the symmetry of the operator:
 * F_k = -1/2 m^T (dA/dx_k) m.  perp, para, rvals, n_tab: the tables the system
 * was created with (their segment slopes are the derivative of the interpolated
 * couplings).  forces: n x 3.  dE_deps (optional, n): dE/d eps_k of the
 * permittivity set diag_index.  Synchronises once. */
int mps_adjoint_forces(mps_system *sys, const double *m, const double *perp, const double *para,
                       const double *rvals, int64_t n_tab, int32_t diag_index, double *forces, double *dE_deps,
                       mps_stream_t stream);

/* ------------------------------------------------------------------------- */
/* Point-dipole pair forces (the HOOMD plugin's kernel)                        */
/* ------------------------------------------------------------------------- */

/* Replaces compute_forces(pos, dip, box, r_cut, prefactor, periodic_z, use_cell_list) of
 * "CPU - HOOMD simulation test/dipole_forces_ext/_dipole_forces_ext.cpp:119-497".
 * pos, dip: n x 3; box: host double[3]; forces: n x 3; pe: n (half of each pair
 * energy on each particle).  Returns MPS_RC_GT_HALF_BOX when r_cut >= L/2 in a
 * periodic axis (the reference's RuntimeError). */
int mps_dipole_forces(const double *pos, const double *dip, int64_t n, const double *box, double r_cut,
                      double prefactor, int32_t periodic_z, double *forces, double *pe, mps_stream_t stream);

/* ------------------------------------------------------------------------- */
/* Allocation-free neighbour list (no counterpart in the reference: its Python */
/* allocates freely).  For callers that must not allocate device memory while */
/* they run, e.g. a simulation engine that owns all device memory and calls a */
/* field/force plugin every time step: cudaMalloc/cudaFree synchronise the    */
/* device and may fail mid-run.                                              */
/* ------------------------------------------------------------------------- */

/* Size of the fixed device scratch array behind mps_neighbor_list_noalloc,
 * resident on every GPU that loads the library until the process exits. */
#define MPS_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* Same result as mps_neighbor_list_count + mps_neighbor_list_fill (the
 * reference's candidate pairs, in its order) without any workspace argument and
 * without allocating: the scratch is a fixed MPS_NOALLOC_SCRATCH_BYTES device
 * array inside the library.  Inputs and outputs are still the caller's:
 * cell (n x 3 int64), p1/p2 with room for max_pairs int64 each.  *n_pairs (host)
 * receives the pair count.  Returns MPS_SCRATCH_LIMIT, before touching the GPU,
 * when mps_neighbor_list_workspace(n, ncell) exceeds the scratch (roughly
 * n > 32,000 particles), and MPS_SCRATCH_LIMIT with *n_pairs set when the pairs
 * do not fit in max_pairs, and MPS_BAD_ARG, also before touching the GPU, when
 * a cell count is below 1 or the cell counts' product overflows.  The first call
 * on a device looks up that device's scratch address; make it before any stream
 * capture.  The call waits for the pair count (data dependent), then queues the
 * fill on `stream` and returns: p1/p2 are ready only in the order of `stream`,
 * and the scratch stays in use until that fill has run.  All calls share the one
 * array: calls whose GPU work overlaps (other streams, other host threads) race,
 * so serialise them. */
int mps_neighbor_list_noalloc(const int64_t *cell, int64_t n, const int64_t *ncell, int64_t *p1, int64_t *p2,
                              int64_t max_pairs, int64_t *n_pairs, mps_stream_t stream);

/* ------------------------------------------------------------------------- */
/* Diagnostics (no counterpart in the reference, which only prints timers at  */
/* EW/capacitance.py:92-108, 367-394).                                         */
/* ------------------------------------------------------------------------- */

/* Number of kernels this library has launched since it was loaded. */
uint64_t mps_kernel_launches(void);

/* enable != 0: every matvec records CUDA events around its stages (slab sum,
 * spread, forward FFT, scale, inverse FFT, contract, real space). */
int mps_system_profile(mps_system *sys, int32_t enable);

/* Accumulated stage times since the last call (synchronises on the recorded
 * events): ms[21] = [float64 stages 0..6, float32 stages 0..6, double-float
 * stages 0..6] in milliseconds, count[3] = matvecs recorded per precision.
 * Resets the accumulators. */
int mps_system_stage_times(mps_system *sys, double *ms, int64_t *count);

/* Drops the process's cache of Green's coefficients and scale tensors (keyed by
 * device, grid, box, xi and eta; shared by systems built on the same grid), so
 * the next system built recomputes its k-space data, as the reference does on
 * every capacitance() call (EW/capacitance.py:385).  Systems that hold
 * coefficients keep them until destroyed.  Host only; no GPU work. */
int mps_kspace_cache_clear(void);

/* Tile depth of the tiled kernels: tile_depth[0] for the float64-width tiles
 * (float64 or double-float spread, whichever ran first, timed by the
 * autotuner), [1] for the float32 tiles (the gradient-form spread -- on the
 * inner grid when the system has one, depth 12 where the grid allows it, not
 * timed -- or the reference-form spread + contract) (0 = not used yet);
 * ms[4] = the timed candidates (depth 4, depth 8) of those kernels,
 * float64-width then float32, -1 where not timed. */
int mps_system_tuning(const mps_system *sys, int32_t *tile_depth, float *ms);

/* GMRES step graphs of a system (no reference counterpart: the reference's
 * GMRES loop, EW/capacitance.py:60-199, runs on the host).  mps_gmres runs the
 * Arnoldi steps of a cycle as one CUDA graph launch -- a while-conditional node
 * whose body is one step (matvec, Gram-Schmidt, Givens update, next basis
 * vector, device-side convergence test) -- once a matvec of that precision and
 * batch width has run outside a capture; the host reads the convergence
 * estimates once per launch instead of once per step.  built = graphs
 * instantiated, failed = configurations whose capture the runtime refused
 * (those keep host-driven steps).  The environment variable
 * MPS_GMRES_GRAPH=0 selects the host-driven steps. */
int mps_system_graphs(const mps_system *sys, int32_t *built, int32_t *failed);

#ifdef __cplusplus
}
#endif

#endif /* MPS_GB300_H */
