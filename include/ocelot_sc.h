/*
 * ocelot_sc.h -- C ABI of the GB300 (sm_103a) 3D space-charge kick.
 *
 * This library replaces the numerical body of Ocelot's space-charge physics
 * process, class SpaceCharge in ocelot/cpbd/sc.py.  Every entry point below
 * names the reference function whose behaviour it reproduces.  Arguments are
 * plain pointers and sizes: device pointers unless stated otherwise, streams
 * as cudaStream_t passed through a void*.  No entry point allocates device
 * memory: the caller owns every buffer, including the workspace sized by
 * sc_workspace_bytes().  All calls are asynchronous on the given stream
 * unless stated otherwise; errors in arguments are reported synchronously by
 * the return code, errors found on the device are latched in the workspace
 * and read with sc_read_status().
 *
 * Return codes: SC_OK or one of the SC_ERR_* values; sc_last_error() gives a
 * message for the calling thread's last failure.
 */
#ifndef OCELOT_SC_H
#define OCELOT_SC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SC_ABI_VERSION 1

/* mode of a plan: a precision, optionally OR-ed with FP32-form options */
#define SC_FP64 0 /* plain form: FP64 end to end, matches sc.py to 1e-10 */
#define SC_FP32 1 /* precision form: FP32 deposit/FFT/gather, FP64 accumulation into
                     rparticles; by default the charge is accumulated exactly in
                     64-bit fixed point and the Green's function far from the
                     origin uses a cancellation-free 4th-order multipole form */
#define SC_FP32_SORTED_DEPOSIT 0x10 /* FP32 form: radix sort + Kahan segment sums */
#define SC_FP32_EXACT_IGF 0x20      /* FP32 form: FP64 8-corner IGF on every cell */
#define SC_FP32_SPECTRAL_FIELDS 0x40 /* FP32 form: forward-difference fields taken in Fourier space */

/* status codes */
#define SC_OK 0
#define SC_ERR_ARG 1         /* invalid argument (checked on the host) */
#define SC_ERR_CUDA 2        /* a CUDA runtime call failed */
#define SC_ERR_WORKSPACE 3   /* workspace missing, too small or not initialised */
#define SC_ERR_DEGENERATE 4  /* zero or non-finite beam extent / charge (device) */
#define SC_ERR_NONFINITE 5   /* non-finite particle coordinate or momentum (device) */
#define SC_ERR_UNSUPPORTED 6 /* grid too large for the FFT plan */
#define SC_ERR_TIMEOUT 7     /* a device-side wait gave up after its iteration limit */
#define SC_ERR_OOM 8         /* host or device memory for the library's own buffers could not be allocated */

typedef struct sc_plan sc_plan; /* opaque, host-side only */

/* ---- plan / workspace ------------------------------------------------- */

/* Plan for a mesh of nx*ny*nz cells (SpaceCharge.nmesh_xyz, sc.py:94) in the
 * given mode (SC_FP64, or SC_FP32 with options).  Each n must be >= 4 (the reference divides the extent by
 * n-3, sc.py:179).  Holds sizes, FFT radix plans, launch shapes and the stream
 * and events of the Green's-function branch -- no device memory; everything a
 * kick needs besides stream operations is set up here, so kicks can be
 * recorded in a CUDA graph. */
int sc_plan_create(sc_plan** plan, int nx, int ny, int nz, int mode);
void sc_plan_destroy(sc_plan* plan);
/* padded FFT lengths chosen for the linear convolution (each >= 2n-1) */
int sc_plan_fft_shape(const sc_plan* plan, int* mx, int* my, int* mz);

/* Bytes of device workspace for kicks of up to n_max particles. */
int64_t sc_workspace_bytes(const sc_plan* plan, int64_t n_max);
/* Prepare a freshly allocated workspace (twiddle tables, empty Green's-function
 * cache, cleared status).  Required once after allocation. */
int sc_workspace_init(const sc_plan* plan, void* ws, size_t ws_bytes, void* stream);
/* Synchronous: waits for the stream, returns the status latched on the
 * device by the last call using this workspace (SC_OK when none). */
int sc_read_status(const sc_plan* plan, void* ws, void* stream);

/* Where an intermediate of the last call lives in the workspace, for
 * inspection: the NGP charge grid of el_field (sc.py:193), the potential
 * (sc.py:168), the field grids Ex/Ey/Ez (sc.py:195-200), all [nx][ny][nz];
 * the cell keys (sc.py:192) as uint32[n].  Grids are double for an SC_FP64
 * plan and float for SC_FP32.  Offsets do not depend on n except for keys.
 * A kick of an SC_FP32_SPECTRAL_FIELDS plan leaves the potential out (its
 * field octs do not need it) unless SC_PARAM_RECORD_FIELD is set.
 * SC_REGION_STATUS is the int that sc_read_status returns (the last kick's
 * status) and SC_REGION_FIRST_ERROR an int holding the first non-OK status of
 * any earlier kick since sc_workspace_init: a device-resident loop of many
 * kicks copies the two asynchronously instead of synchronising per kick. */
#define SC_REGION_QGRID 0
#define SC_REGION_PHI 1
#define SC_REGION_EX 2
#define SC_REGION_EY 3
#define SC_REGION_EZ 4
#define SC_REGION_KEYS 5
#define SC_REGION_STATUS 6
#define SC_REGION_FIRST_ERROR 7
/* With SC_PARAM_RECORD_FIELD set: the field each particle of the last kick
 * was kicked with -- the trilinear samples of Ex, Ey, Ez at the particle
 * before the gamma0 factor (sc.py:201-204) -- as 3 rows of nX = n rounded up
 * to a multiple of 4 (double for SC_FP64, float for SC_FP32). */
#define SC_REGION_FIELD 8
/* SC_REGION_IGF: the cell integrals of the Green's function of the last
 * call, [nx][ny][nz] in the plan's precision (FP32 form: the hybrid table of
 * 8-corner FP64 differences near the origin, the line form across and the
 * multipole form beyond; the table is rebuilt only when the mesh step
 * changes). */
#define SC_REGION_IGF 9
int sc_workspace_region(const sc_plan* plan, int64_t n_max, int region, int64_t* offset, int64_t* bytes);

/* ---- the kick ---------------------------------------------------------- */

/* SpaceCharge.apply(p_array, zstep)  -- sc.py:208-251.
 *   rparticles: device, float64, row r of particle i at rparticles[r*ld + i]
 *               (the 6xN MAD coordinates x, x', y, y', tau, delta),
 *               rewritten in place like xp_2_xxstg_mad (coord_transform.py:16-54);
 *   q:          device, float64[n] macro-particle charges (ParticleArray.q_array);
 *   energy_gev: reference energy (ParticleArray.E);
 *   zstep:      kick length in metres; 0 returns immediately (sc.py:210-212);
 *   mesh_scale / mesh_shift: the two draws of random_mesh (sc.py:174-175,
 *               184-185), or NaN when random_mesh is off.
 * On a device-side error the particles are left unchanged. */
int sc_kick(sc_plan* plan, void* ws, size_t ws_bytes, double* rparticles, int64_t ld,
            const double* q, int64_t n, double energy_gev, double zstep,
            double mesh_scale, double mesh_shift, void* stream);

/* ---- many beams at once ------------------------------------------------ */

/* One kick for each of many beams, each with its own plan (mesh), workspace
 * and particles, in ONE launch per stage: every stage kernel runs over a
 * device work table whose prefix rows map each block to a beam and to its
 * block within that beam's grid.  A beam keeps the grids, reductions and
 * arithmetic of a single sc_kick, so its result is bit-identical to
 * sc_kick's alone; the number of launches per batched kick (15) does not
 * depend on the number of beams.  No counterpart in the reference, whose
 * track() kicks one beam at a time (ocelot/cpbd/track.py:476-478): this is
 * the multi-beam entry of the same SpaceCharge.apply (sc.py:208-251).
 *
 * Requirements: every plan is SC_FP32 without SC_FP32_SORTED_DEPOSIT (the
 * exact fixed-point deposit), each beam has its own plan and initialised
 * workspace, and no two beams share a workspace or particles.  A beam with
 * zstep == 0 is not kicked (sc.py:210-212); if it carries a transport map it
 * stays in the table for sc_tmap_batched alone (its workspace and energy are
 * then not used), otherwise it is left out. */
typedef struct sc_batch sc_batch;
typedef struct sc_beam {
    sc_plan* plan;
    void* ws;
    size_t ws_bytes;
    double* rparticles;     /* device float64 [6][ld] */
    int64_t ld;
    const double* q;        /* device float64 [n] */
    int64_t n;
    double energy_gev;
    double zstep;
    double mesh_scale;      /* NAN unless random_mesh */
    double mesh_shift;
    const double* tmap;     /* host float64[42]: R (row-major) then B, for sc_tmap_batched; or NULL */
} sc_beam;

/* A batch of up to max_beams beams.  Allocates its work table (device and
 * pinned host, about 1 KB per beam) and a second stream with two events. */
int sc_batch_create(sc_batch** out, int max_beams);
void sc_batch_destroy(sc_batch* batch);
/* Validates the beams and uploads the work table with an asynchronous copy
 * on `stream`.  Waits (on the host) only for the copy of the previous call.
 * Not allowed during stream capture.  On any error the batch keeps the table
 * it had.  Once a kick or transport of this batch has been recorded in a CUDA
 * graph, the graph's launches (number of beams, blocks per stage, shared
 * memory) are fixed: a table of another shape -- other particle counts or
 * meshes, a beam more or less, a kick length set to zero -- is refused with
 * SC_ERR_ARG, and those beams are kicked with a new batch.  Tables of the same
 * shape (new kick lengths, energies, maps, buffers) are accepted. */
int sc_batch_set(sc_batch* batch, const sc_beam* beams, int nbeams, void* stream);
/* Kicks every beam of the table currently set (stream-ordered after the
 * upload).  Capturable in a CUDA graph; a replay kicks the beams of the
 * table resident at replay time (of the shape recorded, see sc_batch_set).
 * Fails with SC_ERR_WORKSPACE, launching nothing, when a beam's plan had its
 * workspace initialised again (sc_workspace_init) after sc_batch_set: set the
 * table again.  A graph recorded before that still holds the old workspace;
 * set the table again before replaying it.  Device errors latch in each
 * beam's workspace (sc_read_status). */
int sc_kick_batched(sc_batch* batch, void* stream);
/* Kernels launched by the last sc_kick_batched (0 before the first). */
int sc_batch_launches(const sc_batch* batch);
/* Stage timing of batched kicks, as sc_profile_enable / sc_profile_read of a
 * plan (the same SC_NSTAGES stages, summed over the beams of each launch);
 * the events sit between the launches, so kicks timed this way run a little
 * slower.  No counterpart in the reference. */
int sc_batch_profile_enable(sc_batch* batch, int enable);
int sc_batch_profile_read(sc_batch* batch, float* ms /* [SC_NSTAGES] */);
/* rparticles <- R . rparticles + B for every beam of the table that was set
 * with a map (sc_beam.tmap), in one launch: the transport before the kick of
 * a tracking step (TransferMap.mul_p_array, transfer_map.py:40-50), with the
 * arithmetic of sc_tmap_apply.  Capturable like sc_kick_batched. */
int sc_tmap_batched(sc_batch* batch, void* stream);

/* ---- stages, mirroring SpaceCharge's public methods ------------------- */

/* SpaceCharge.el_field(X, Q, gamma, nxyz) -- sc.py:170-205.
 *   X: device float64 [n][3] rotated positions; modified in place as the
 *      reference modifies it (z scaled by gamma);  exyz: device float64 [n][3]. */
int sc_el_field(sc_plan* plan, void* ws, size_t ws_bytes, double* X, const double* q, int64_t n,
                double gamma, double mesh_scale, double mesh_shift, double* exyz, void* stream);

/* SpaceCharge.potential(q, steps) -- sc.py:135-168.
 *   qgrid, phi: device float64 [nx][ny][nz]. */
int sc_potential(sc_plan* plan, void* ws, size_t ws_bytes, const double* qgrid,
                 double hx, double hy, double hz, double* phi, void* stream);

/* SpaceCharge.sym_kernel(q.shape, steps) -- sc.py:109-133, always FP64.
 *   kern: device float64 [nx][ny][nz]. */
int sc_sym_kernel(sc_plan* plan, void* ws, size_t ws_bytes, double hx, double hy, double hz,
                  double* kern, void* stream);

/* The table of sc_sym_kernel computed without any workspace or device
 * allocation.  No counterpart in the reference: it serves callers that cannot
 * allocate device memory where they need the table -- processes whose device
 * memory is reserved up front by another allocator or a fixed budget, and
 * latency-critical loops that must not call cudaMalloc/cudaFree (which can
 * synchronise the device).  The scratch is one static device array of
 * SC_SYM_KERNEL_STATIC_MAX_CORNERS doubles (4 MiB), held by every GPU that
 * loads the library until the process exits; meshes need
 * (nx+1)(ny+1)(nz+1) <= SC_SYM_KERNEL_STATIC_MAX_CORNERS (64^3 fits), larger
 * ones are rejected with SC_ERR_UNSUPPORTED.  The first call on a device
 * looks up the array's device address, so make it before any stream capture.
 * That address is kept for the life of the process: after cudaDeviceReset on
 * a device it is stale, so do not call this entry point on that device again.
 * All calls share the array: calls that overlap on the GPU (other streams or
 * host threads) race -- keep them on one stream.
 *   kern: device float64 [nx][ny][nz]. */
#define SC_SYM_KERNEL_STATIC_MAX_CORNERS 524288
int sc_sym_kernel_static(int nx, int ny, int nz, double hx, double hy, double hz, double* kern,
                         void* stream);

/* Stable LSD radix sort of 32-bit cell keys with their particle indices: the
 * summation order of the deposit, equal to numpy.argsort(keys, kind='stable')
 * -- it replaces the sequential np.bincount of sc.py:193.
 *   keys_in: device uint32[n], each < 2^key_bits; keys_out, perm_out: device uint32[n]. */
int64_t sc_sort_workspace_bytes(int64_t n, int key_bits);
int sc_sort_keys(const uint32_t* keys_in, int64_t n, int key_bits, uint32_t* keys_out,
                 uint32_t* perm_out, void* ws, size_t ws_bytes, void* stream);

/* ---- transport between kicks ------------------------------------------ */

/* TransferMap.mul_p_array -- transformations/transfer_map.py:40-50:
 * rparticles <- R . rparticles + B for a first-order map.
 *   R: host float64[36] row-major (already tilt-rotated, first_order_params.py:26-28);
 *   B: host float64[6]. */
int sc_tmap_apply(const double* R, const double* B, double* rparticles, int64_t ld, int64_t n,
                  void* stream);

/* The transport steps of a tracking loop kept on the device: the same map as
 * sc_tmap_apply, taken from a device table of maps -- map i is
 * table[i*42 .. i*42+35] (R, row-major) and table[i*42+36 .. i*42+41] (B) --
 * at i = *counter (a device int; out of range: no transport), after which
 * *counter is incremented, in stream order.  The maps are the element slices
 * Navigator.get_map builds between two kicks (ocelot/cpbd/navi.py:406-434),
 * composed, applied as TransferMap.apply does; with the index on the device,
 * one recorded step (this call, then sc_kick) replays for every step. */
int sc_tmap_apply_indexed(const double* table, int* counter, int nmaps, double* rparticles,
                          int64_t ld, int64_t n, void* stream);

/* Second-order maps: SecondTM.t_apply of drift/quadrupole slices
 * (ocelot/cpbd/transformations/second_order.py:31-38, SecondOrderMult.numpy_apply,
 * ocelot/cpbd/tm_utils.py:54-55): x <- R.x + T:xx, then x <- x + B.
 *   maps: DEVICE float64[nmaps * SC_MAP2_DOUBLES], map m at maps + m*SC_MAP2_DOUBLES:
 *         R[36] row-major (tilt applied), B[6], then Tc[6][21], the coefficient
 *         of x_j x_k (j <= k, pairs in lexicographic order) in output i, i.e.
 *         T[i,j,k] + T[i,k,j] for j < k and T[i,j,j] on the diagonal.
 * The maps are applied in order with each particle's coordinates kept in
 * registers (second-order maps do not compose exactly, so the slices of a
 * step are not multiplied together). */
#define SC_MAP2_DOUBLES 168
int sc_tmap2_apply(const double* maps, int nmaps, double* rparticles, int64_t ld, int64_t n, void* stream);

/* The second-order transport of a tracking loop kept on the device: the maps
 * [first[s], first[s+1]) of a device table at s = *counter (a device int;
 * out of range: no transport), then *counter += 1, in stream order, so that
 * one recorded step replays for every step (as sc_tmap_apply_indexed).
 *   first: DEVICE int32[nsteps + 1]. */
int sc_tmap2_apply_step(const double* maps, const int* first, int* counter, int nsteps, double* rparticles,
                        int64_t ld, int64_t n, void* stream);

/* Slices of a tracking step that pass RF cavities: each record of the table
 * (SC_MAP2_DOUBLES doubles) is either a map as in sc_tmap2_apply
 * (kinds[m] = SC_SLICE_MAP; a first-order map has Tc = 0) or a cavity slice
 * (kinds[m] = SC_SLICE_CAVITY), CavityTM.map4cav
 * (ocelot/cpbd/transformations/cavity.py:29-128): x <- R.x + B with the
 * slice's first-order matrix (elements/cavity_atom.py:93-179, tilt applied),
 * then from the coordinates before it
 *   x5 <- x5 E beta0 / D + A (cos(-x4 beta0 k + phi) - cos(phi)),
 *   x4 <- x4 + T566 x5^2 + T556 x4 x5 + T555 x4^2
 * with the record's doubles 42..55: E (energy at the slice start, GeV), beta0,
 * D = E1 beta1, A = V beta0 / D, k = 2 pi f / c, phi [rad], cos(phi), T566,
 * T556, T555, a flag that is 0 when the energy after the slice is not
 * positive (then only the T566 term is applied and x5 keeps R.x + B),
 * RN(1/D), sin(phi), and a flag that is non-zero when R's non-zero entries lie
 * in the x, y and longitudinal 2x2 blocks.  The host computes the scalars in
 * the reference's order of operations; the device divides by D as a product
 * with RN(1/D) and one FMA correction, and evaluates cos near phi as
 * cos(phi) + cos(phi)(cos d - 1) - sin(phi) sin d (d = arg - phi, |d| <= 1/4;
 * cos(arg) otherwise) -- within an ulp or two of the reference's values.
 *   kinds: DEVICE int32[nmaps]. */
#define SC_SLICE_MAP 0
#define SC_SLICE_CAVITY 1
/* A map (as SC_SLICE_MAP) whose non-zero entries lie in the pattern of an untilted quadrupole or drift without
 * offsets -- R: (0,0) (0,1) (1,0) (1,1) (2,2) (2,3) (3,2) (3,3) (4,4) (4,5) (5,5); Tc: outputs 0,1 at the pairs
 * (0,5) (1,5), outputs 2,3 at (2,5) (3,5), output 4 at (0,0) (0,1) (1,1) (2,2) (2,3) (3,3) (5,5) -- or, for
 * SC_SLICE_MAP_DRIFT, of a drift -- R: (0,0) (0,1) (1,1) (2,2) (2,3) (3,3) (4,4) (4,5) (5,5); Tc: output 0 at
 * (1,5), output 2 at (3,5), output 4 at (1,1) (3,3) (5,5).  Evaluated over the pattern only, with the same result
 * as SC_SLICE_MAP for finite coordinates; the caller guarantees the pattern. */
#define SC_SLICE_MAP_PLANAR 2
#define SC_SLICE_MAP_DRIFT 3
/* A first-order map (Tc = 0) whose R lies in the SC_SLICE_MAP_PLANAR pattern. */
#define SC_SLICE_MAP_LINEAR 4
int sc_slices_apply(const double* maps, const int* kinds, int nmaps, double* rparticles, int64_t ld, int64_t n,
                    void* stream);

/* The slices [first[s], first[s+1]) at s = *counter, then *counter += 1, in
 * stream order (the transport of a device-resident tracking loop through a
 * line with cavities; as sc_tmap2_apply_step). */
int sc_slices_apply_step(const double* maps, const int* kinds, const int* first, int* counter, int nsteps,
                         double* rparticles, int64_t ld, int64_t n, void* stream);

/* Beam moments after a tracking step: get_envelope (ocelot/cpbd/beam/analysis.py:27-226) without dispersion
 * correction, the statistics track() takes after every step (ocelot/cpbd/track.py:466-486).  Writes slot
 * s = *counter (counter NULL: slot 0; out of [0, nslots): nothing) of a DEVICE table out[nslots][SC_MOMENTS]:
 *   [0] particles counted, [1] mean and [2] standard deviation of tau over all particles (only with bounds),
 *   [3..8] means of x, y, px', py', tau, p, [9..20] central moments xx, xpx, pxpx, yy, ypy, pypy, tautau,
 *   xy, pxpy, xpy, ypx, pp, with px' = px f, py' = py f, f = 1 - p - p^2/2 + px^2/2 + py^2/2.
 * use_bounds: only the particles with m + lo s <= tau <= m + hi s count (get_envelope's bounds, in units of
 * the standard deviation s of tau around its mean m).  One launch (two with bounds): sums shifted by the
 * first particle's values, so the central moments carry no cancellation; the sums are deterministic.  scratch: DEVICE, sc_moments_scratch_bytes() bytes, zero-filled once before the first call,
 * not shared by concurrent calls. */
#define SC_MOMENTS 21
int64_t sc_moments_scratch_bytes(void);
int sc_moments(const double* rparticles, int64_t ld, int64_t n, const int* counter, int nslots, int use_bounds,
               double lo, double hi, double* out, void* scratch, void* stream);

/* ---- stage timing (benchmarking) --------------------------------------- */

/* Stages of sc_kick: MAD->lab frame (coord_transform.py:57-96,
 * sc.py:224-239), mesh extent (sc.py:171-186), NGP keys (sc.py:187-192),
 * radix sort, deposit (sc.py:193), IGF table (sc.py:109-133) and Green
 * spectrum (sc.py:142-149,164) -- these two on a second stream, beside keys,
 * sort and deposit --, the wait for them, convolution (sc.py:150-168), field
 * grids (sc.py:195-200), gather + kick + back-transform (sc.py:201-251). */
#define SC_NSTAGES 11
/* When enabled, sc_kick records a CUDA event on its stream before the first
 * stage and after each stage.  Host call; creates or destroys the events. */
int sc_profile_enable(sc_plan* plan, int enable);
/* Synchronous (waits for the last event): milliseconds of each stage of the
 * last profiled sc_kick, and the number of kernels that call launched. */
int sc_profile_read(sc_plan* plan, float* ms /* [SC_NSTAGES] */, int* n_launches);
const char* sc_profile_stage_name(int stage);
/* Number of kernels the plan's last sc_kick launched (host bookkeeping, no
 * synchronisation). */
int sc_kick_launches(const sc_plan* plan);

/* Launch shapes a plan may choose without changing any result (the
 * autotuner's knobs, ocelot_gb300/tuning.py).  No counterpart in the
 * reference, whose only knob is the FFT thread count (sc.py:152-160).
 *   SC_PARAM_KICK_VARIANT: tiling of the FP32 gather + kick, 0 ..
 *     SC_KICK_NVARIANTS - 1, described by sc_kick_variant; every tiling runs
 *     the same per-particle arithmetic, so the kick is bit-identical.  A new
 *     plan starts with the tiling measured fastest on large beams. 
 * Set between kicks (not during a stream capture that uses the plan). */
#define SC_PARAM_KICK_VARIANT 0
/*   SC_PARAM_RECORD_FIELD: 1 makes every kick also store the field at each
 *     particle (SC_REGION_FIELD), for error measurements; the FP32 form then
 *     runs its direct-access kick loop (same arithmetic, same particles). */
#define SC_PARAM_RECORD_FIELD 1
/*   SC_PARAM_FFT_PLANE_FWD / SC_PARAM_FFT_PLANE_INV: 1 (default) runs the z
 *     and y transforms of one x plane in one block where the plane fits
 *     shared memory (one launch per direction, 64 blocks on a 64^3 mesh); 0
 *     runs them as separate passes of many smaller blocks.  The lines go
 *     through the same transform code either way: identical results. */
#define SC_PARAM_FFT_PLANE_FWD 2
#define SC_PARAM_FFT_PLANE_INV 3
/*   SC_PARAM_FFT_COLS_X / SC_PARAM_FFT_COLS_Y: lines (columns of the work
 *     grid) per block of the x pass and of the separate y passes: 2, 4, 8 or
 *     16, or 0 (default) for as many as fit, up to 16.  Fewer columns per
 *     block take less shared memory, so more blocks share an SM.  The lines
 *     are independent: identical results.  A batched kick also caps them so
 *     that four blocks share an SM. */
#define SC_PARAM_FFT_COLS_X 4
#define SC_PARAM_FFT_COLS_Y 5
#define SC_KICK_NVARIANTS 21
int sc_plan_set_param(sc_plan* plan, int param, int value);
int sc_plan_get_param(const sc_plan* plan, int param, int* value);
/* Tile (particles), tile buffers, particles per thread and blocks per SM of a
 * kick variant. */
int sc_kick_variant(int variant, int* tile, int* stages, int* particles_per_thread, int* blocks_per_sm);

/* Failure detection of the bulk-copy waits.  The frame, extent and kick
 * kernels of the FP32 form stream particle rows through shared memory with
 * bulk copies and wait for each on an mbarrier with an iteration limit
 * (2^20 tries of about 1 us); a wait that runs out latches SC_ERR_TIMEOUT in
 * the workspace state, waits once more (full limit) for its copies still in
 * flight and returns, so the context stays usable and sc_read_status reports
 * the error.  This sets the limit of one kernel (SC_WAIT_FRAME, _EXTENT,
 * _KICK) or of all three (-1) for this plan's later kicks; tries < 0 restores
 * the default, larger values are clamped to it.  Tries = 0 makes the first
 * wait give up at once -- the way the tests exercise the timeout path without
 * a fault or a hang.  A timeout in the frame or extent leaves the particles
 * unchanged; in the kick, tiles whose wait gave up are not written (tiles of
 * other blocks may be).  No counterpart in the reference (it has no device
 * waits). */
#define SC_WAIT_FRAME 0
#define SC_WAIT_EXTENT 1
#define SC_WAIT_KICK 2
int sc_plan_set_wait_limit(sc_plan* plan, int kernel, long long tries);

/* ---- misc -------------------------------------------------------------- */
const char* sc_last_error(void);
int sc_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* OCELOT_SC_H */
