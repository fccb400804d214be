/*
 * gimic_gb300: C ABI of the GB300 (sm_103a) GIMIC current-density path.
 *
 * Two layers are exported from libgimic_gb300.so:
 *
 *  1. Drop-in replacements of the reference's own C interface, same names
 *     and argument meaning:
 *       - src/libgimic/gimic_interface.h:9-17 (gimic_init ... gimic_calc_modj,
 *         implemented in src/libgimic/gimic_interface.f90:26-163);
 *       - src/libgimic/gausspoints.h:10-12 (mkgausspoints,
 *         gimic_get_gauss_points; src/libgimic/gausspoints.f90:12-29).
 *     Like the reference they keep one module-global molecule and stop the
 *     process (exit status 1, message on stderr) on fatal input errors.
 *
 *  2. A context API (gg_*) with status codes, batched point evaluation on
 *     device or host buffers, plane integrals and explicit precision control.
 *     Every gg_* function returns 0 on success or a negative GG_E* code; the
 *     message is available from gg_last_error().
 *
 * Conventions: coordinates in Bohr; current tensors are 3x3 column-major,
 * t(m,b) = dj_m/dB_b at index m + 3b (src/libgimic/jtensor.F90:148-237);
 * currents in atomic units (gg_au2si converts to nA/T).
 */
#ifndef GIMIC_GB300_H
#define GIMIC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference-compatible interface --------------------------------------
 * Replaces src/libgimic/gimic_interface.h:9-17.  r is one point (3 doubles),
 * jt a 3x3 column-major tensor, jv = jt . B with B from gimic_set_magnet. */
void gimic_init(const char *molfile, const char *densfile);  /* gimic_interface.f90:26-70 */
void gimic_finalize(void);                                   /* :72-78 */
void gimic_set_uhf(int *uhf);                                /* :80-86; reloads XDENS if changed after init */
void gimic_set_magnet(const double *b);                      /* :88-91 */
void gimic_set_spin(const char *spin);                       /* :93-114 alpha|beta|total|spindens */
void gimic_set_screening(const double *thrs);                /* :116-119; used by the next gimic_init */
void gimic_calc_jtensor(const double *r, double *jt);        /* :121-139 */
void gimic_calc_jvector(const double *r, double *jv);        /* :141-151 */
void gimic_calc_modj(const double *r, double *mj);           /* :153-163 (stops: not implemented, as in the reference) */

/* Replaces src/libgimic/gausspoints.h:10-12: composite Gauss-Legendre points
 * and weights, npts/order panels, placed on [0, b - a] exactly as
 * setup_gauss_data (src/libgimic/gaussint.f90:267-319) does. */
void gimic_get_gauss_points(double *a, double *b, int *npts, int *order, double *pts, double *wgts);
void mkgausspoints(double *a, double *b, int *npts, int *order, double *pts, double *wgts);

/* ---- context API ---------------------------------------------------------- */
#define GG_OK 0
#define GG_EINVAL (-1)     /* bad argument */
#define GG_EIO (-2)        /* input file missing or malformed */
#define GG_ECUDA (-3)      /* CUDA runtime error (no device, launch failure) */
#define GG_ENOMEM (-4)     /* device allocation failed */
#define GG_ETIMEDOUT (-5)  /* a device-side wait gave up (kernel reported an error) */
#define GG_EUNSUPPORTED (-6)

#define GG_PREC_FP64 0     /* plain FP64 path: SIMT DGEMM + FP64 assembly */
#define GG_PREC_SPLIT16 1  /* split-FP16 x3 tcgen05 GEMM, FP32 accumulate, double-float combine (default) */

typedef struct gg_ctx gg_ctx;

/* Reads MOL (INTGRL) and XDENS as gimic_init does (basis.f90:29-86,
 * dens.f90:56-127); screening <= 0 disables screening.  Uses the current CUDA
 * device.  On failure *out is NULL and gg_last_error(NULL) has the reason. */
int gg_ctx_create(const char *molfile, const char *xdens, int uhf, double screening, gg_ctx **out);
/* As gg_ctx_create, with the basis choice of the gimic.inp keyword
 * Advanced.spherical (src/fgimic/gimic.F90:85-87, src/gimic.in:79): with
 * spherical != 0 the XDENS blocks are over the spherical functions (2l+1 per
 * shell, m = -l..l, the integer-rescaled solid harmonics of
 * src/libgimic/cao2sao.f90:153-235) and the basis values are their
 * projections (bfeval.f90:116-117).  The projection is folded into the
 * densities once (D_cart = po^T D_sph po), so evaluation costs the same as
 * for the Cartesian basis.  Standard (non-TURBOMOLE) component order only;
 * returns GG_EIO with a message otherwise. */
int gg_ctx_create_ex(const char *molfile, const char *xdens, int uhf, double screening, int spherical,
                     gg_ctx **out);
/* The projection of one shell of angular momentum l (0..5) used by
 * gg_ctx_create_ex: (2l+1) x (l+1)(l+2)/2 row-major, rows m = -l..l, columns
 * the standard Cartesian component order (the operator of mkc2sop and
 * renorm, src/libgimic/cao2sao.f90:173-235; for l >= 4 the reference's
 * term-by-term assignment is kept).  No device work. */
int gg_spherical_projection(int l, double *out);
int gg_ctx_destroy(gg_ctx *ctx);
const char *gg_last_error(const gg_ctx *ctx);

int gg_set_spin(gg_ctx *ctx, const char *spin);            /* alpha|beta|total|spindens */
int gg_set_magnet(gg_ctx *ctx, const double b[3]);
int gg_get_magnet(const gg_ctx *ctx, double b[3]);
int gg_set_screening(gg_ctx *ctx, double thrs);            /* takes effect on the next evaluation */
int gg_set_flags(gg_ctx *ctx, int giao, int diamag, int paramag);  /* Advanced.GIAO/diamag/paramag */
int gg_set_precision(gg_ctx *ctx, int mode);               /* GG_PREC_* */
/* Points per device pass (scratch size), at least 128; 0 restores the
 * default.  By default the split path takes the largest power of two from
 * 2^18 to 2^21 whose scratch (two pipeline slots of 4 nbf + 128 bytes per
 * point) fits 16 GiB; the FP64 path at most 16,384. */
int gg_set_max_batch(gg_ctx *ctx, int64_t npts);
/* Split path: order the points into compact tiles and skip, per tile, the
 * shells that are screened for all of its points (on by default; results do
 * not change, only the work skipped). */
int gg_set_tile_screening(gg_ctx *ctx, int enable);
/* Split path with tile screening: issue only the main (hi*hi) product of
 * the split for K blocks whose basis values stay below 2^-14 of every
 * point's row bound in the tile (on by default).  The two cross products of
 * such a block add at most one fp32 rounding of the main product's largest
 * terms; the error against the FP64 path is unchanged.  Which blocks qualify
 * depends on a tile's points, so with it on a point's result can differ in
 * the last bits between batch splits; off, every batch split and the tile
 * screening itself give bit-identical results. */
int gg_set_cross_skip(gg_ctx *ctx, int enable);
/* Internal order of the shells (and so of the basis functions and density
 * rows/columns).  mode 1 (the default, set at creation): shells grouped by
 * screening radius, atoms along a nearest-neighbour tour, when that activates
 * fewer tiles' K blocks and column chunks than the file order; mode 0: the
 * file order.  Results are the same up to rounding.  gg_get_shell_order
 * returns the mode and, when order is not NULL, order[k] = file index of the
 * shell at position k (nshells entries, see gg_basis_info). */
int gg_set_shell_order(gg_ctx *ctx, int mode);
int gg_get_shell_order(const gg_ctx *ctx, int *mode, int *order);

/* nbf: contracted Cartesian functions; turbomole: 1 if the MOL file has the
 * TURBOMOLE header (component order gtodefs.f90:108-123). */
int gg_basis_info(const gg_ctx *ctx, int *nbf, int *natoms, int *nshells, int *turbomole);
int gg_atoms(const gg_ctx *ctx, double *coords /* natoms x 3 */, double *charges);

/* Current tensors at n points.  pts: n x 3; jt: n x 9 (column-major 3x3);
 * rho: n (electron density of the selected spin case, or null); divt: n x 3,
 * divt[b] = sum_m d t(m,b)/d r_m (null to skip; needs GIAO, dia and para on).
 * Buffers may be host or device memory (not mixed host/device for inputs vs
 * outputs is fine).  stream: a cudaStream_t or null for the default stream.
 * Returns after the results are complete. */
int gg_jtensor_batch(gg_ctx *ctx, const double *pts, int64_t n, double *jt, double *rho, double *divt, void *stream);
/* Property quadratures over a molecular grid (replaces get_property,
 * src/fgimic/jfield.f90:584-929): the current tensor is evaluated at the n
 * points pts (n x 3, Bohr) with weights wgt (n), and for the field along -x,
 * -y and -z the code sums
 *   nuclear shielding of every centre K (ncentres x 3 coordinates, Bohr):
 *     sigma_a(K) = sum_i w_i 1e6 f_i ((r_i - R_K) x j_i)_a,
 *     f_i = -1 / |r_i - R_K|^3 / 137.0359998^2   (ppm),
 *   magnetizability: chi_a = sum_i w_i 0.5 (r_i x j_i)_a   (au),
 * separately over nblocks consecutive blocks of points of block_npts[l]
 * points each (the per-atom blocks of the grid generator, nelpts.info; null
 * or nblocks <= 0: one block).  Outputs, host memory:
 *   sigma[(K * nb + l) * 5 + q], chi[l * 5 + q], nb = number of blocks,
 *   q = 0..2 the diagonal sums, 3 and 4 the positive and negative parts of
 *   sum_a (value at the point) * w_i.
 * Summing over l gives the reference's totals; the per-block sums divided by
 * 3 are its printed atom contributions. */
int gg_properties(gg_ctx *ctx, const double *pts, const double *wgt, int64_t n, const double *centres, int ncentres,
                  const int64_t *block_npts, int nblocks, double *sigma, double *chi, void *stream);

/* The same with fp32 outputs (each value computed in fp64 and rounded once),
 * for grids too large to keep in fp64 (no reference counterpart; the
 * reference writes its fields through Fortran real(8) arrays). */
int gg_jtensor_batch_f32(gg_ctx *ctx, const double *pts, int64_t n, float *jt, float *rho, float *divt,
                         void *stream);

/* jv = t . B with B the context's magnetic field (jtensor.F90:125-135). */
int gg_jvector_batch(gg_ctx *ctx, const double *pts, int64_t n, double *jv, void *stream);

/* Product grid r(i,j,k) = origin + x1_i basv1 + x2_j basv2 + x3_k basv3
 * (src/fgimic/grid.f90:498-511) with quadrature weights per axis. */
typedef struct {
  double origin[3];
  double basv[9];        /* basv[3*d + c]: component c of axis d; axis 2 is the plane normal */
  int npts[3];
  const double *pts[3];  /* host arrays, npts[d] each */
  const double *wgt[3];
  double radius;         /* points farther than this from the grid centre get weight 0 */
} gg_grid;

/* Plane integral (integral.f90:50-186, :190-324, :414-511) with the context's
 * magnetic field.  out[0..2] current (total, positive, negative), out[3..5]
 * signed modulus (total, positive, negative), out[6] ACID sum (the reference
 * prints sqrt(out[6])).  All in atomic units. */
int gg_plane_integral(gg_ctx *ctx, const gg_grid *grid, double out[7], void *stream);

/* A batch of planes in one device pass (bond-current profile scans, as the
 * reference's jobscripts/src/current-profile-header:132-146 drive plane by
 * plane): out is nplanes x 7 in the layout of gg_plane_integral. */
int gg_plane_integrals(gg_ctx *ctx, const gg_grid *grids, int nplanes, double *out, void *stream);

/* gg_plane_integrals in two halves, so that one host thread can queue many
 * molecules' passes before waiting for any (the reference runs one gimic
 * process per molecule and slice, jobscripts/src/current-profile-header:
 * 112-146).  _enqueue queues the pass on `stream` and returns without
 * waiting; the host work of the next molecule then overlaps this one's
 * device work.  _collect waits for that pass, checks the device error word,
 * copies the nplanes x 7 sums to out and, when ms is given, stores the
 * stream time from the pass's first to its last operation (waits for work
 * queued ahead of it excluded).  Between the two calls the context must not
 * evaluate anything else (its scratch holds the pending pass); a second
 * _enqueue before _collect is rejected. */
int gg_plane_integrals_enqueue(gg_ctx *ctx, const gg_grid *grids, int nplanes, void *stream);
int gg_plane_integrals_collect(gg_ctx *ctx, double *out, double *ms);

/* Plane passes of many molecules in one contraction launch: the batched
 * form of the reference's per-molecule, per-slice job loop
 * (jobscripts/src/current-profile-header:132-146, each slice a run of
 * integral.f90:50-186).  Molecule m (context ctxs[m], all distinct, on one
 * device, split-FP16 precision, the same GIAO/dia/para flags) integrates
 * nplanes[m] planes grids[m]; the points, ordering, tile screening and basis
 * evaluation of every molecule's whole pass come first, then one persistent
 * contraction kernel takes the tiles of all molecules from one queue (job
 * order: 0 as given, 1 the most expensive molecules, points x nbf^2, first),
 * then each molecule's reduction.  out receives sum(nplanes) x 7 sums in
 * molecule order, laid out as gg_plane_integrals; mol_ms (optional, nmol)
 * the time from the contraction's start to the completion of each
 * molecule's last tile.  From the second call with the same contexts and
 * layouts on, the whole batch is replayed as one CUDA graph.  Blocking. */
int gg_plane_integrals_batch(gg_ctx *const *ctxs, const gg_grid *const *grids, const int *nplanes, int nmol,
                             int order, double *out, double *mol_ms, void *stream);

/* Composite quadrature (gaussint.f90:267-319); type 0 Gauss-Legendre,
 * 1 Gauss-Lobatto.  Returns GG_EINVAL if npts is not a multiple of order or
 * the Newton iteration fails. */
int gg_gauss_data(double a, double b, int order, int npts, int type, double *pts, double *wgts);

double gg_au2si(double au);  /* au -> nA/T (globals.f90 au2si) */

/* Self-timing: with profiling on, every kernel group the context launches is
 * bracketed by CUDA events on its stream; gg_profile_read returns the summed
 * milliseconds and launch counts per group since gg_profile(ctx, 1), and the
 * number of kernels launched.  No reference counterpart (the reference times
 * itself with etime, src/libgimic/timer.f90). */
#define GG_PROF_BASIS 0  /* fp32 basis evaluation + fp16 split of the point operand */
#define GG_PROF_TC 1     /* tcgen05 contraction + fused current-tensor epilogue */
#define GG_PROF_FP64 2   /* plain FP64 path (basis, DGEMM, assembly) */
#define GG_PROF_PLANE 3  /* plane quadrature reduction */
#define GG_PROF_ORDER 4  /* spatial ordering of the points and tile screening */
#define GG_NPROF 5
int gg_profile(gg_ctx *ctx, int enable);
int gg_profile_read(const gg_ctx *ctx, double ms[GG_NPROF], int64_t launches[GG_NPROF], int64_t *total_kernels);
/* GEMM work since gg_profile(ctx, 1), in blocks of 128 points x 224 columns x
 * 64 (three fp16 products each): issued after tile screening, and the count
 * a dense contraction would have issued. */
int gg_profile_blocks(const gg_ctx *ctx, int64_t *issued, int64_t *dense);
/* Of the issued blocks since gg_profile(ctx, 1), those that also issued the
 * two cross products of the split (the others, gg_set_cross_skip, issued
 * only the main product). */
int gg_profile_cross(const gg_ctx *ctx, int64_t *cross);

/* Self-tests of the failure paths (no counterpart in the reference, whose
 * Fortran stops the process on an error).  Every device-side wait of the
 * library is bounded: on expiry the kernel records a code in the context's
 * device error word and returns, and the next host check reports
 * GG_ETIMEDOUT; the context stays usable.  Neither entry faults, traps or
 * hangs the GPU.
 * gg_selftest_wait_timeout: runs a one-thread kernel that waits on an
 *   mbarrier nothing arrives at, with a limit of limit_ms (0 < limit_ms <=
 *   2000), through the pipeline kernels' own wait routine; returns
 *   GG_ETIMEDOUT (error code 100 in gg_last_error) and, when waited_ms is
 *   given, the time the wait took.
 * gg_selftest_fail_next: records `code` (nonzero) in the device error word,
 *   as a failed wait of another thread would; the next evaluation's kernels
 *   leave their pipelines without work and the call returns GG_ETIMEDOUT with
 *   that code, after which the word is clear again. */
int gg_selftest_wait_timeout(gg_ctx *ctx, double limit_ms, double *waited_ms, void *stream);
int gg_selftest_fail_next(gg_ctx *ctx, int code);

/* Integration proposal network (no counterpart in the reference, which
 * integrates on fixed grids, src/fgimic/integral.f90:50-511).  A 5 -> 64 ->
 * 64 -> 1 multilayer perceptron with SiLU activations predicts ln|j| at a
 * point of an integration plane; the adaptive plane integrator refines a
 * quadtree of Gauss-Lobatto panels where it predicts large, fast-varying
 * currents.  Parameters are gg_mlp_nparams() fp32 values laid out as
 * W1[64][5] b1[64] W2[64][64] b2[64] W3[64] b3.  Every array is device
 * memory; non-device pointers are rejected with GG_EINVAL.
 *
 * gg_mlp_features: the five inputs for n points pts (n x 3, Bohr) with
 *   in-plane coordinates uv (n x 2, Bohr): u/8, v/8, ln of the distances to
 *   the nearest and second-nearest nucleus, and the local shell-exponent
 *   density log10(1e-6 + sum_s sqrt(a_s) exp(-a_s d_s^2)) / 3 (a_s: smallest
 *   exponent of shell s); feats is n x 5 fp32.
 * gg_mlp_grad: gradient of the mean squared error (1/n) sum (y_i - t_i)^2
 *   over the n samples x (n x 5) with targets t, written to grad (overwritten),
 *   and the loss itself when loss is not null.
 * gg_mlp_adam: one Adam step (bias-corrected, step counted from 1).
 * gg_mlp_infer: predictions y (n) with bf16-rounded weights and activations. */
int gg_mlp_nparams(void);
int gg_mlp_features(gg_ctx *ctx, const double *pts, const double *uv, int64_t n, float *feats, void *stream);
int gg_mlp_grad(const float *params, const float *x, const float *target, int64_t n, float *grad, float *loss,
                void *stream);
int gg_mlp_adam(float *params, const float *grad, float *m, float *v, float lr, float beta1, float beta2, float eps,
                int step, void *stream);
int gg_mlp_infer(const float *params, const float *x, int64_t n, float *y, void *stream);

/* Evaluation without device allocation (no counterpart in the reference).
 * For callers that cannot let a library call cudaMalloc or cudaFree: host
 * applications that budget all device memory themselves, and time-critical
 * loops where an allocation would stall the device.  Same results as
 * gg_jtensor_batch on the split-FP16 path, but the per-point scratch lives in
 * a fixed 32 MiB static device array (plus a 4-byte static counter, held on
 * every GPU where the library's device code is loaded, until the process
 * exits), so n is limited to
 * floor((32 MiB - 768) / (4 * kpad + 4)) points, kpad = nbf rounded up to 64
 * (10,908 points for nbf 720); larger n is rejected with GG_EINVAL and a
 * message.  All buffers must be device memory, and the context must already
 * be prepared for its current spin case by one gg_jtensor_batch call (that
 * call allocates the device tables).  The first call on a device looks up the
 * array's address, so make it before any stream capture.  Every call reuses
 * the same array: calls that overlap on the GPU (other streams, other
 * contexts, other threads) race on it and must be serialised by the caller.
 * As on the other split-FP16 entry points nbf is at most 4096, and a plane
 * pass queued with gg_plane_integrals_enqueue must be collected first.  With
 * gg_profile on, its two kernels are timed as the basis and contraction
 * groups and counted as dense (unscreened) GEMM blocks. */
int gg_jtensor_batch_noalloc(gg_ctx *ctx, const double *pts, int64_t n, double *jt, double *rho, double *divt,
                             void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GIMIC_GB300_H */
