// Internal declarations shared by the translation units of libocelot_sc.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/ocelot_sc.h"

namespace ocsc {

// ---------------------------------------------------------------------------
// complex helpers (float2 / double2)
// ---------------------------------------------------------------------------
template <typename R> struct CT;
template <> struct CT<float> { using T = float2; };
template <> struct CT<double> { using T = double2; };
template <typename R> using Cx = typename CT<R>::T;

template <typename R> __host__ __device__ __forceinline__ Cx<R> cx(R a, R b) { Cx<R> c; c.x = a; c.y = b; return c; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
// multiply by -i (forward) or +i (inverse)
template <typename C> __device__ __forceinline__ C cmul_mi(C a) { C c; c.x = a.y; c.y = -a.x; return c; }
template <typename C> __device__ __forceinline__ C cmul_pi(C a) { C c; c.x = -a.y; c.y = a.x; return c; }

// ---------------------------------------------------------------------------
// constants: the expressions of ocelot/common/globals.py:13-24 evaluated in
// IEEE double on the host, so they are bit-identical to the reference's.
// ---------------------------------------------------------------------------
struct PhysConst {
    double pi, m_e_eV, m_e_GeV, epsilon_0;
};
PhysConst phys_const();

// ---------------------------------------------------------------------------
// device-resident state of one workspace (first bytes of the workspace)
// ---------------------------------------------------------------------------
struct ScState {
    // velocity frame (sc.py:224-239); T[i][j] = component i of basis vector j
    double T[3][3];
    double Pav, gamma0, beta0;
    double kxy, kz;              // cdT*(1-beta0^2) and cdT (sc.py:244-248)
    // mesh (sc.py:171-186)
    double steps[3];
    double xoff[3];
    double isteps[3];            // 1/steps
    double phi_denom;            // 4*pi*eps0*hx*hy*hz (sc.py:167)
    double phi_norm;             // 1/(Mx*My*Mz) of the inverse FFT
    float phi_scalef;            // (float)(phi_norm / phi_denom): the FP32 form's potential scale
    // Green's-function cache: spacing of the spectrum held in the workspace
    double igf_h[3];
    // FP32 copies of the per-kick constants, written once by the finalizes
    float Tf[3][3];
    float g0f, ig0f, kxyf, kzf;
    float stepsf[3], istepsf[3], xofff[3];
    int igf_rebuild;             // 1 when the current call rebuilds it
    int status;                  // SC_OK or a device-side SC_ERR_*
    int ws_magic;                // set by sc_workspace_init
    // exact fixed-point deposit of the FP32 form: charge units of 2^-qfix_shift
    double qfix_scale;           // 2^qfix_shift
    float qfix_inv;              // 2^-qfix_shift
    int qfix_shift;
    // near box of the hybrid Green's function (cells with all indices below
    // it use the FP64 8-corner formula)
    int igf_box[3];
    // cells long along z (hz the largest step): the transverse near box of
    // the line form (igf_line_of)
    int igf_line;
    int igf_tbox[2];
    unsigned int done_frame;     // blocks finished, for the last-block reductions
    unsigned int done_extent;
    unsigned int kick_next;      // tiles claimed by the gather + kick (reset by the frame finalize)
    int frame_timeout;           // a frame block's bulk-copy wait gave up (the finalize reports it)
    int check_code;              // checked builds: first failed index check (kernel code)
    int first_error;             // first non-OK status of any kick since sc_workspace_init
    long long check_index;       // ... and the offending index (checked builds)
};
static_assert(sizeof(ScState) <= 512, "the state must fit the 512 bytes the static IGF scratch reserves");
constexpr int WS_MAGIC = 0x5c6b0e11;

// Near box of the hybrid Green's function: along each axis the cells with
// index below ceil(5 hmax / h) + 1.  Every cell outside it is at least
// 5 hmax from the origin, where the 4th-order multipole form of the cell
// integral is within 5e-8 of the exact integral (checked against an
// extended-precision IGF).  Written into the state once per kick by the
// kernel that sets the mesh step.
// Cells long along z (hz >= hx, hy; every relativistic beam whose bunch is
// not much shorter than it is wide): the near box along z keeps its
// ceil(5 hz / hz) + 1 = 6 cells, but across it only the cells within
// ceil(5 ht / h) + 1 of the axis (ht = max(hx, hy)) need the 8-corner
// formula.  The cells of the first six z planes farther out are at least
// 5 ht from the z axis, where the line form of the cell integral (exact
// along z, Gauss-Legendre across) is within FP32 rounding of the exact
// integral (igf_line in sc_green.cu).  axis 0 or 1; FP32 arithmetic with a
// relative margin of 2^-20 (the box is at most one cell larger than exact).
__device__ __forceinline__ bool igf_line_of(const double (&h)[3]) { return h[2] >= h[0] && h[2] >= h[1]; }
__device__ __forceinline__ int igf_tbox_of(const double (&h)[3], int axis, int n) {
    const float ht = (float)fmax(h[0], h[1]);
    const float v = 5.0f * ht / (float)h[axis] * (1.0f + 0x1p-20f);
    const int b = v >= (float)n ? n : (int)ceilf(v) + 1;
    return b > n ? n : b;
}

__device__ __forceinline__ void igf_box_of(const double (&h)[3], int nx, int ny, int nz, int (&b)[3]) {
    const double hm = fmax(h[0], fmax(h[1], h[2]));
    const int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
        const double v = 5.0 * hm / h[a];
        b[a] = v >= (double)n[a] ? n[a] : (int)ceil(v) + 1;
        if (b[a] > n[a]) b[a] = n[a];
    }
}

// host-computed scalars of one kick
struct KickParams {
    int64_t n, ld;
    int64_t nX;                          // row stride of the 3-row grid-coordinate array (n rounded up to 4)
    int nx, ny, nz;
    int Mx, My, Mz;
    double gamref, betaref, pref, grbr;  // grbr = gamref*betaref
    // RN(1/x) of the four above and of m2, for correctly rounded division by them (Markstein)
    double r_gamref, r_betaref, r_pref, r_grbr, r_m2;
    double cdT;                          // zstep / betref
    double mesh_scale, mesh_shift;       // NaN when unused
    double m_e_eV, m2;                   // m_e_eV and m_e_eV**2
    double four_pi_eps0;                 // 4*pi*epsilon_0
    double phi_norm;                     // 1/(Mx*My*Mz) of the inverse FFT
    // FP32 copies for the FP32 form
    float gamref_f, betaref_f, grbr_f, pref_f, ipref_f, m_f, m2_f;
    float igrbr2_f;                      // 1/(gamref*betaref)^2
    // iteration limits of the bulk-copy waits of the frame, extent and kick
    // kernels (MBAR_WAIT_LIMIT unless a test lowers them, sc_plan_set_wait_limit)
    unsigned wait_limit[3];
};

// ---------------------------------------------------------------------------
// FFT geometry and radix plans
// ---------------------------------------------------------------------------
constexpr int MAX_STAGES = 8;
struct RadixPlan {
    int L;
    int nst;
    int r[MAX_STAGES];
};
bool make_radix_plan(int L, RadixPlan* p);
// Line stride (in complex elements) of every FFT line buffer in shared
// memory: room for the padded layout of the intermediate Stockham stages
// (element i at i + i/8) plus one element, so that lines start on
// different banks
__host__ __device__ constexpr int fft_ls(int L) { return L + L / 8 + 1; }
int choose_fft_length(int n);  // smallest supported length >= 2n-1, 0 if none

// ---------------------------------------------------------------------------
// workspace layout (offsets in bytes from the workspace base)
// ---------------------------------------------------------------------------
struct Layout {
    size_t state, tw_x, tw_y, tw_z;              // twiddles (Cx<R>[M])
    size_t part_frame, part_ext;                 // per-block partial sums (double)
    size_t xp;                                   // FP64: 6 x n lab coordinates
    size_t X;                                    // 3 x n grid coordinates (R)
    size_t keys, sort_keys, sort_perm, sort_q, sort_tmp_k, sort_tmp_v, sort_hist, sort_tot;
    size_t qgrid, phi, ex, ey, ez;               // [nx][ny][nz] (R)
    size_t exq, eyq, ezq;                        // FP32 form: [nx][ny][nz] gather octs (8 floats, 32-byte aligned)
    size_t cell_start, cell_end;                 // [nx*ny*nz] uint32 run bounds (adjacent)
    size_t qfix;                                 // [nx*ny*nz] int64 fixed-point charge (FP32 form)
    size_t igf_ig;                               // (nx+1)(ny+1)(nz+1) double
    size_t igf_k1;                               // nx*ny*nz (R; double storage size)
    size_t green_s1, green_s2, green;            // spectrum passes (R)
    size_t W;                                    // complex work grid nx*My*Kz
    // spectral fields (FP32 with SC_FP32_SPECTRAL_FIELDS): the forward-difference
    // factors 1 - exp(2 pi i k / M) per axis (Cx<R>[M]) and two more work grids
    size_t dt_x, dt_y, dt_z, W2, W3;
    size_t total;
};

struct Plan {
    int nx, ny, nz, prec;
    bool sorted_deposit;  // FP64 always; FP32 with SC_FP32_SORTED_DEPOSIT
    bool exact_igf;       // FP64 always; FP32 with SC_FP32_EXACT_IGF
    bool spectral;        // FP32 with SC_FP32_SPECTRAL_FIELDS
    int Mx, My, Mz;
    RadixPlan rx, ry, rz;
    int key_bits;
    int sm_count;
    int part_blocks;   // blocks of the per-particle reduction kernels
    unsigned wait_limit[3];  // KickParams::wait_limit of this plan's kicks
    int kick_variant;        // tiling of the FP32 gather + kick (sc_particles.cu, SC_KICK_VARIANTS)
    int record_field;        // the kick also stores the field at each particle (SC_REGION_FIELD)
    int fft_plane_fwd;       // 1: plane-fused z + y forward passes where the plane fits, 0: separate passes
    int fft_plane_inv;       // 1: plane-fused y + z inverse passes where the plane fits, 0: separate passes
    int fft_cols_x;          // columns per block of the x pass (0: as many as fit, up to 16)
    int fft_cols_y;          // columns per block of the separate y passes (0: as many as fit, up to 16)
};
// tile, tile buffers, particles per thread and blocks per SM of kick variant v (0 if v is out of range)
int kick_variant_info(int v, int* tile, int* stages, int* ppt, int* minb);
int default_kick_variant();

Layout make_layout(const Plan& p, int64_t n);

// ---------------------------------------------------------------------------
// launchers (each returns cudaError_t of the launch)
// ---------------------------------------------------------------------------
cudaError_t launch_init_workspace(const Plan& p, const Layout& L, char* ws, cudaStream_t s);

// per-particle stages (sc_particles.cu)
cudaError_t launch_frame(const Plan& p, const Layout& L, char* ws, const KickParams& kp,
                         const double* rp, cudaStream_t s);
cudaError_t launch_extent(const Plan& p, const Layout& L, char* ws, const KickParams& kp,
                          const double* rp, const double* q, cudaStream_t s);
// rp: the particles (exact recomputation of near-face keys in the FP32 form), or nullptr
// FP32 form without the sorted deposit: also accumulates q into the
// fixed-point grid (the deposit), zeroed first unless qfix_zeroed (the
// FP32 frame kernel of the same kick zeroes it)
cudaError_t launch_keys(const Plan& p, const Layout& L, char* ws, const KickParams& kp, const double* rp,
                        const double* q, cudaStream_t s, bool qfix_zeroed = false);
cudaError_t launch_gather_kick(const Plan& p, const Layout& L, char* ws, const KickParams& kp,
                               double* rp, cudaStream_t s);
// el_field entry: extent over a given X[n][3] with a given gamma, and gather to exyz
cudaError_t launch_extent_xyz(const Plan& p, const Layout& L, char* ws, const KickParams& kp,
                              double* X, const double* q, double gamma, cudaStream_t s);
cudaError_t launch_gather_xyz(const Plan& p, const Layout& L, char* ws, const KickParams& kp,
                              double* exyz, cudaStream_t s);

// sort + deposit (sc_sort.cu)
size_t sort_scratch_bytes(int64_t n, int key_bits);
int sort_blocks(int64_t n);  // blocks of a sort of n keys (rows of its digit histogram)
int sort_passes(int key_bits);
// With q_src set, the last pass writes q_src[index] (as double or float) into
// q_out instead of the permutation.
cudaError_t launch_sort(const uint32_t* keys_in, int64_t n, int key_bits, uint32_t* keys_out,
                        uint32_t* perm_out, uint32_t* tmp_k, uint32_t* tmp_v, uint32_t* hist,
                        uint32_t* tot, cudaStream_t s, const double* q_src = nullptr, void* q_out = nullptr,
                        bool q_float = false);
cudaError_t launch_deposit(const Plan& p, const Layout& L, char* ws, const double* q, int64_t n,
                           cudaStream_t s);

// Green's function (sc_green.cu)
cudaError_t launch_igf(const Plan& p, const Layout& L, char* ws, cudaStream_t s);
cudaError_t launch_igf_h(const Plan& p, const Layout& L, char* ws, double* kern_out, double hx, double hy,
                         double hz, cudaStream_t s);
cudaError_t launch_set_mesh(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double hx, double hy,
                            double hz, cudaStream_t s);
cudaError_t launch_green_spectrum(const Plan& p, const Layout& L, char* ws, cudaStream_t s);

// convolution + field grids (sc_fft.cu)
// qfix: the fixed-point charge grid of the FP32 form's exact deposit (then
// qgrid_in receives the scaled grid), or nullptr
// part: CONV_ALL, or CONV_FORWARD (z and y forward passes: they need only the
// charge grid) and then CONV_REST (the passes that need the Green spectrum)
enum ConvPart { CONV_ALL = 0, CONV_FORWARD = 1, CONV_REST = 2 };
cudaError_t launch_convolve(const Plan& p, const Layout& L, char* ws, const void* qgrid_in,
                            void* phi_out, cudaStream_t s, const long long* qfix = nullptr, int part = CONV_ALL,
                            bool fields = false, bool want_phi = true);
cudaError_t launch_field_grids(const Plan& p, const Layout& L, char* ws, cudaStream_t s);
// kernels launch_convolve(CONV_ALL) launches for this plan
int convolve_launches(const Plan& p);

// first-order map (sc_tmap.cu)
cudaError_t launch_tmap(const double* R, const double* B, double* rp, int64_t ld, int64_t n,
                        cudaStream_t s);
cudaError_t launch_tmap2(const double* maps, const int* kinds, int nmaps, double* rp, int64_t ld, int64_t n,
                         cudaStream_t s);
cudaError_t launch_tmap2_step(const double* maps, const int* kinds, const int* first, int* counter, int nsteps,
                              double* rp, int64_t ld, int64_t n, cudaStream_t s);
cudaError_t launch_moments(const double* rp, int64_t ld, int64_t n, const int* counter, int nslots, int use_bounds,
                           double lo, double hi, double* out, void* scratch, cudaStream_t s);
size_t moments_scratch_bytes();
cudaError_t launch_tmap_indexed(const double* table, int* counter, int nmaps, double* rp, int64_t ld,
                                int64_t n, cudaStream_t s);

// ---------------------------------------------------------------------------
// Batched kicks (sc_kick_batched): one launch per stage over many beams.
//
// Every kernel body takes the coordinates of its block within its beam's
// grid (VBlk).  A plain launch passes the hardware's; a batched launch runs
// one 1D grid that is the concatenation of every beam's grid for that stage,
// and each block finds its beam in a prefix table of block counts.  The
// per-beam grids are the ones the plain launches use, so a beam's arithmetic
// -- reduction trees included -- is the same in a batch as alone.
// ---------------------------------------------------------------------------
struct VBlk {
    int x, y, nx, ny;
};
__device__ __forceinline__ VBlk hw_vblk() {
    return VBlk{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y};
}

enum BatchStage {
    BS_PART = 0,   // frame, extent, keys, kick (one block per PT particles, capped)
    BS_IGF_C,      // IGF corners
    BS_IGF_D,      // IGF cell differences
    BS_GREEN_Z,    // spectrum S1
    BS_GREEN_Y,    // spectrum S2
    BS_GREEN_X,    // spectrum S3
    BS_FFT_Z,      // F1
    BS_FFT_Y,      // F2
    BS_FFT_X,      // F3 (x forward, Green multiply, x inverse)
    BS_FFT_YI,     // B2 (with spectral fields: two groups of blocks, W and the x-differenced W2)
    BS_FFT_ZI,     // B1 (with spectral fields: four groups, the potential and Ex, Ey, Ez)
    BS_FIELD,      // field quads
    BS_TMAP,       // transport map (sc_tmap_batched): also the beams without a kick this step
    BS_COUNT
};

struct BatchBeam {
    char* ws;
    double* rp;
    const double* q;
    KickParams kp;
    Layout L;
    Plan p;
    int vec_rp, vec_rpq;              // 16-byte row accesses allowed: rparticles / rparticles and q
    int has_tm;                       // a transport map to apply before the kick (sc_tmap_batched)
    double tm[42];                    // R (row-major), then B
    int fft_nc, fft_tky, fft_tkx;     // convolution tiling
    int green_nc, green_tky, green_tkx;
    int gx[BS_COUNT], gy[BS_COUNT];   // this beam's grid per stage
};

// beam of this block: the last b with start[b] <= blockIdx.x (start[nb] = total)
__device__ __forceinline__ int batch_beam(const int* __restrict__ start, int nb) {
    const int bid = (int)blockIdx.x;
    int lo = 0, hi = nb;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(start + mid) <= bid) lo = mid;
        else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ VBlk batch_vblk(const int* __restrict__ start, int b, int gx, int gy) {
    const int local = (int)blockIdx.x - __ldg(start + b);
    return VBlk{local % gx, local / gx, gx, gy};
}

// batched stage launchers; start = the stage's prefix row (nb + 1 entries)
enum BatchPartKernel { BP_FRAME, BP_EXTENT, BP_KEYS, BP_KICK };
cudaError_t launch_batch_particles(BatchPartKernel k, const BatchBeam* beams, const int* start, int nb, int blocks,
                                   cudaStream_t s);
cudaError_t launch_batch_igf(const BatchBeam* beams, const int* start_c, const int* start_d, int nb, int blocks_c,
                             int blocks_d, cudaStream_t s);
cudaError_t launch_batch_green(const BatchBeam* beams, const int* sz, const int* sy, const int* sx, int nb,
                               const int blocks[3], const size_t smem[3], cudaStream_t s);
cudaError_t launch_batch_convolve(const BatchBeam* beams, const int* sz, const int* sy, const int* sx,
                                  const int* syi, const int* szi, int nb,
                                  const int blocks[5], const size_t smem[3], cudaStream_t s, int part = CONV_ALL);
cudaError_t launch_batch_field(const BatchBeam* beams, const int* start, int nb, int blocks, cudaStream_t s);
cudaError_t launch_batch_tmap(const BatchBeam* beams, const int* start, int nb, int blocks, cudaStream_t s);
// host-side tiling of one beam (sets the tiling fields and grids of B)
void batch_fft_tiling(BatchBeam& B, size_t smem[3]);
void batch_green_tiling(BatchBeam& B, size_t smem[3]);
int batch_particle_blocks(const Plan& p, int64_t n);
int batch_igf_blocks(const Plan& p, int diff);
// opt the batched kernels in to the device's largest dynamic shared memory
cudaError_t prepare_batch_fft();
cudaError_t prepare_batch_green();

inline size_t align_up(size_t v, size_t a = 256) { return (v + a - 1) / a * a; }

// Programmatic dependent launch: every kernel of this library is launched
// with launch(), which lets its blocks be scheduled while the previous
// kernel of the stream drains, and begins with pdl_wait(), which holds it
// until that kernel has completed and its memory writes are visible.  (A
// kernel launched without the attribute passes pdl_wait() at once.)
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                          Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Opt a kernel in to the device's largest dynamic shared memory, once per
// kernel (a registry keyed by the kernel's address), so that launches made
// later -- including those recorded in a CUDA graph capture -- issue no
// attribute calls.
cudaError_t smem_opt_in(const void* kernel, size_t bytes);
template <typename K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return smem_opt_in(reinterpret_cast<const void*>(kernel), bytes);
}
// opts every kernel of a plan in (called when the plan is created)
cudaError_t prepare_fft_kernels(const Plan& p);
cudaError_t prepare_green_kernels(const Plan& p);
cudaError_t prepare_particle_kernels();

// ---------------------------------------------------------------------------
// bulk (TMA) copies between global and shared memory.  Loads complete on an
// mbarrier (expect_tx / complete_tx); stores are bulk groups.  Every wait has
// an iteration limit: a wait that gives up returns false and the caller
// records SC_ERR_TIMEOUT instead of spinning on.
// ---------------------------------------------------------------------------
constexpr unsigned MBAR_WAIT_LIMIT = 1u << 20;  // tries of ~1 us at most each

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the async proxy (then __syncthreads)
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// true once the phase with the given parity has completed; false when the
// limit ran out first
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned limit = MBAR_WAIT_LIMIT) {
    const uint32_t a = smem_u32(bar);
    for (unsigned it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(1000u)
            : "memory");
        if (done) return true;
    }
    return false;
}
// global -> shared, bytes a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst_smem)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// shared -> global (same rules), part of the current bulk group
__device__ __forceinline__ void bulk_store(void* dst, const void* src_smem, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src_smem)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// all but the newest N bulk groups have finished reading shared memory
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
// every bulk group has completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Per-thread asynchronous copies global -> shared (cp.async): 8 bytes, both
// addresses 8-byte aligned; src_bytes 0 fills the 8 bytes with zeros.  A
// thread's copies form groups (commit) and wait_group<N> waits until at most
// N of the calling thread's newest groups are still in flight -- a wait on
// the thread's own copies only, which complete like ordinary loads.
__device__ __forceinline__ void async_copy8(void* dst_smem, const void* src, unsigned src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst_smem)), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// orders this thread's shared-memory writes before later async-proxy reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// records the calling thread's error message (sc_last_error) and returns code
int sc_report(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));

// Index checks of checked builds (-DSC_CHECKED): a failed check records the
// kernel code and the index in the state and the access is skipped.
#ifdef SC_CHECKED
#define SC_IDX_OK(st, code, idx, size)                                                          \
    ((long long)(idx) >= 0 && (long long)(idx) < (long long)(size)                            \
         ? true                                                                                 \
         : (atomicCAS(&const_cast<ScState*>(st)->check_code, 0, (code)) == 0                   \
                ? ((const_cast<ScState*>(st)->check_index = (long long)(idx)), false)           \
                : false))
#else
#define SC_IDX_OK(st, code, idx, size) true
#endif

}  // namespace ocsc
