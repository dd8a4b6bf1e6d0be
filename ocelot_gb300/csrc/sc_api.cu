// C ABI of libocelot_sc: plans, workspace layout, argument checking and the
// launch sequence of each entry point (see include/ocelot_sc.h).
#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "sc_common.cuh"
#include "sc_fft_dev.cuh"

namespace ocsc {

cudaError_t launch_igf_h(const Plan& p, const Layout& L, char* ws, double* kern_out, double hx, double hy,
                         double hz, cudaStream_t s);
cudaError_t launch_set_mesh(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double hx, double hy,
                            double hz, cudaStream_t s);

cudaError_t smem_opt_in(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::unordered_map<const void*, size_t> opted;
    std::lock_guard<std::mutex> lock(mu);
    auto it = opted.find(kernel);
    if (it != opted.end() && it->second >= bytes) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev))) return e;
    // the dynamic limit is what the kernel's static shared memory leaves
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, kernel))) return e;
    const size_t room = (size_t)optin > fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
    if (bytes > room) return cudaErrorInvalidValue;
    if ((e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room))) return e;
    opted[kernel] = room;
    return cudaSuccess;
}

PhysConst phys_const() {
    // ocelot/common/globals.py:13-24
    PhysConst c;
    c.pi = 3.141592653589793;
    const double speed_of_light = 299792458.0;
    const double q_e = 1.6021766208e-19;
    const double m_e_kg = 9.10938215e-31;
    c.m_e_eV = m_e_kg * pow(speed_of_light, 2.0) / q_e;
    c.m_e_GeV = c.m_e_eV / 1e+9;
    const double mu_0 = 4 * c.pi * 1e-7;
    c.epsilon_0 = 1 / mu_0 / pow(speed_of_light, 2.0);
    return c;
}

// The smallest length 2^k or 3 * 2^k (8 .. 512) that holds the linear
// convolution of n cells (M >= 2n - 1): 96 cells take 192 rather than 256.
int choose_fft_length(int n) {
    const int need = 2 * n - 1;
    int best = 0;
    for (int L = 8; L <= 512; L *= 2)
        if (L >= need) {
            best = L;
            break;
        }
    for (int L = 12; L <= 384; L *= 2)
        if (L >= need) {
            if (!best || L < best) best = L;
            break;
        }
    return best;
}

bool make_radix_plan(int L, RadixPlan* p) {
    p->L = L;
    p->nst = 0;
    int rem = L;
    if (rem % 3 == 0) {  // one radix-3 stage first (as plan_radix)
        p->r[p->nst++] = 3;
        rem /= 3;
    }
    while (rem % 8 == 0 && rem > 1) {
        if (p->nst >= MAX_STAGES) return false;
        p->r[p->nst++] = 8;
        rem /= 8;
    }
    while (rem % 4 == 0 && rem > 1) {
        p->r[p->nst++] = 4;
        rem /= 4;
    }
    while (rem % 2 == 0 && rem > 1) {
        p->r[p->nst++] = 2;
        rem /= 2;
    }
    return rem == 1;
}

Layout make_layout(const Plan& p, int64_t n) {
    Layout L;
    const size_t rs = p.prec == SC_FP64 ? 8 : 4, cs = 2 * rs;
    const size_t ncell = (size_t)p.nx * p.ny * p.nz;
    const size_t Kx = p.Mx / 2 + 1, Ky = p.My / 2 + 1, Kz = p.Mz / 2 + 1;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t r = o; o += align_up(bytes ? bytes : 1); return r; };
    L.state = take(sizeof(ScState));
    L.tw_x = take(cs * p.Mx);
    L.tw_y = take(cs * p.My);
    L.tw_z = take(cs * p.Mz);
    L.part_frame = take(8 * 3 * (size_t)p.part_blocks);
    L.part_ext = take(8 * 11 * (size_t)p.part_blocks);
    // n-independent regions first: the Green's-function cache keeps its
    // offset when the same workspace serves kicks of different n
    L.qgrid = take(rs * ncell);
    L.phi = take(rs * ncell);
    L.ex = take(rs * ncell);
    L.ey = take(rs * ncell);
    L.ez = take(rs * ncell);
    L.exq = take(p.prec == SC_FP32 ? 32 * ncell : 0);
    L.eyq = take(p.prec == SC_FP32 ? 32 * ncell : 0);
    L.ezq = take(p.prec == SC_FP32 ? 32 * ncell : 0);
    L.cell_start = take(4 * ncell);
    L.cell_end = take(4 * ncell);
    L.qfix = take(8 * ncell);
    L.igf_ig = take(8 * (size_t)(p.nx + 1) * (p.ny + 1) * (p.nz + 1));
    L.igf_k1 = take(8 * ncell);  // R-typed; sized for double
    L.green_s1 = take(rs * (size_t)p.nx * p.ny * Kz);
    L.green_s2 = take(rs * (size_t)p.nx * Ky * Kz);
    L.green = take(rs * Kx * Ky * Kz);
    L.W = take(cs * (size_t)p.nx * p.My * Kz);
    L.dt_x = take(p.spectral ? cs * p.Mx : 0);
    L.dt_y = take(p.spectral ? cs * p.My : 0);
    L.dt_z = take(p.spectral ? cs * p.Mz : 0);
    L.W2 = take(p.spectral ? cs * (size_t)p.nx * p.My * Kz : 0);
    L.W3 = take(p.spectral ? cs * (size_t)p.nx * p.My * Kz : 0);
    L.xp = take(p.prec == SC_FP64 ? 8 * 6 * (size_t)n : 0);
    L.X = take(rs * 3 * (size_t)((n + 3) / 4 * 4));
    L.keys = take(4 * (size_t)n);
    // the radix sort's buffers: only the sorted deposit uses them
    const size_t ns = p.sorted_deposit ? (size_t)n : 0;
    L.sort_keys = take(4 * ns);
    L.sort_perm = take(4 * ns);
    L.sort_q = take(rs * ns);
    L.sort_tmp_k = take(4 * ns);
    L.sort_tmp_v = take(4 * ns);
    const size_t sb = ns ? (size_t)sort_blocks((int64_t)ns) : 1;
    L.sort_hist = take(p.sorted_deposit ? 4 * 512 * sb : 0);
    L.sort_tot = take(p.sorted_deposit ? 4 * 512 : 0);
    L.total = o;
    return L;
}

// the forward difference f[i] - f[i+1] in Fourier space (the transforms'
// convention X[k] = sum x[n] exp(-2 pi i k n / M)): the factor
// 1 - exp(2 pi i k / M) = 2 sin^2(pi k / M) - i sin(2 pi k / M), in the
// half-angle form that keeps its relative accuracy at small k
template <typename R>
__device__ __forceinline__ Cx<R> diff_factor(int k, int M) {
    double s, c, s2;
    sincospi((double)k / M, &s, &c);
    s2 = sinpi(2.0 * k / M);
    return cx<R>((R)(2.0 * s * s), (R)(-s2));
}

template <typename R>
__global__ void k_init_ws(ScState* st, Cx<R>* tx, int Mx, Cx<R>* ty, int My, Cx<R>* tz, int Mz, Cx<R>* dx,
                          Cx<R>* dy, Cx<R>* dz) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        memset(st, 0, sizeof(ScState));
        st->igf_h[0] = st->igf_h[1] = st->igf_h[2] = NAN;
        st->ws_magic = WS_MAGIC;
    }
    // w_M^m, laid out as fft_lines reads it: entry i holds m = i for the
    // two-step lengths, the stage table's m for the Stockham lengths (entries
    // past its M - R0 hold w_M^i, unused)
    double s, c;
    auto entry = [&](int M) {
        const int m = (uses_two_step<R>(M) || i >= M - next_radix(M)) ? i : stage_tw_exponent(M, i);
        sincospi(2.0 * m / M, &s, &c);
        return cx<R>((R)c, (R)-s);
    };
    if (i < Mx) tx[i] = entry(Mx);
    if (i < My) ty[i] = entry(My);
    if (i < Mz) tz[i] = entry(Mz);
    if (dx) {
        if (i < Mx) dx[i] = diff_factor<R>(i, Mx);
        if (i < My) dy[i] = diff_factor<R>(i, My);
        if (i < Mz) dz[i] = diff_factor<R>(i, Mz);
    }
}

cudaError_t launch_init_workspace(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    int m = p.Mx > p.My ? p.Mx : p.My;
    m = m > p.Mz ? m : p.Mz;
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    if (p.prec == SC_FP64)
        launch(k_init_ws<double>, (m + 255) / 256, 256, 0, s, st, (double2*)(ws + L.tw_x), p.Mx, (double2*)(ws + L.tw_y),
                                                          p.My, (double2*)(ws + L.tw_z), p.Mz, (double2*)nullptr,
                                                          (double2*)nullptr, (double2*)nullptr);
    else
        launch(k_init_ws<float>, (m + 255) / 256, 256, 0, s, st, (float2*)(ws + L.tw_x), p.Mx, (float2*)(ws + L.tw_y),
                                                         p.My, (float2*)(ws + L.tw_z), p.Mz,
                                                         p.spectral ? (float2*)(ws + L.dt_x) : (float2*)nullptr,
                                                         (float2*)(ws + L.dt_y), (float2*)(ws + L.dt_z));
    return cudaGetLastError();
}

template <typename A, typename B>
__global__ void k_convert(const A* __restrict__ a, B* __restrict__ b, size_t n) {
    pdl_wait();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = (B)a[i];
}

}  // namespace ocsc

using namespace ocsc;

// events: main stream 0..9 (before frame, after frame, extent, keys, sort,
// deposit, join, convolve, field, kick); side stream 10..12 (start, after
// igf, after green)
constexpr int NEV = 14;

struct sc_plan {
    Plan p;
    const void* ws_ready;  // workspace initialised by sc_workspace_init for this plan
    size_t ws_ready_bytes;
    cudaEvent_t ev[NEV];
    bool profiling;
    int last_launches;
    cudaStream_t side;     // the Green's-function build runs here, beside the deposit
    cudaEvent_t fork, join;
    int* status_host;      // pinned: the status word is read with an asynchronous copy
};

static const char* kStageNames[SC_NSTAGES] = {"frame", "extent", "keys", "sort", "deposit",
                                              "igf", "green", "join_wait", "convolve", "field", "kick"};

static inline void mark(sc_plan* plan, int i, cudaStream_t s) {
    if (plan->profiling) cudaEventRecord(plan->ev[i], s);
}

static thread_local std::string g_err;

static int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
static int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

namespace ocsc {
int sc_report(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
}  // namespace ocsc

static int cuda_fail(cudaError_t e, const char* where) {
    return fail(e == cudaErrorMemoryAllocation ? SC_ERR_OOM : SC_ERR_CUDA, "%s: %s (%s)", where,
                cudaGetErrorString(e), cudaGetErrorName(e));
}

#define SC_CUDA(call, where)                          \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, where); \
    } while (0)

static int check_ws(const sc_plan* plan, const void* ws, size_t ws_bytes, int64_t n) {
    if (!ws) return fail(SC_ERR_WORKSPACE, "workspace is NULL");
    const Layout L = make_layout(plan->p, n);
    if (ws_bytes < L.total)
        return fail(SC_ERR_WORKSPACE, "workspace of %zu bytes is smaller than the %zu needed for n=%lld", ws_bytes,
                    L.total, (long long)n);
    if (plan->ws_ready != ws || plan->ws_ready_bytes != ws_bytes)
        return fail(SC_ERR_WORKSPACE, "workspace was not initialised for this plan (call sc_workspace_init)");
    return SC_OK;
}

static KickParams make_params(const Plan& p, int64_t n, int64_t ld, double energy_gev, double zstep,
                              double mesh_scale, double mesh_shift) {
    const PhysConst c = phys_const();
    KickParams kp;
    memset(&kp, 0, sizeof kp);
    kp.n = n;
    kp.ld = ld;
    kp.nX = (n + 3) / 4 * 4;
    kp.nx = p.nx; kp.ny = p.ny; kp.nz = p.nz;
    kp.Mx = p.Mx; kp.My = p.My; kp.Mz = p.Mz;
    // sc.py:214-216 and coord_transform.py:19-20,61
    kp.gamref = energy_gev / c.m_e_GeV;
    kp.betaref = sqrt(1 - pow(kp.gamref, -2.0));
    kp.pref = c.m_e_eV * sqrt(pow(kp.gamref, 2.0) - 1);
    kp.grbr = kp.gamref * kp.betaref;
    kp.cdT = zstep / kp.betaref;
    kp.mesh_scale = mesh_scale;
    kp.mesh_shift = mesh_shift;
    kp.m_e_eV = c.m_e_eV;
    kp.m2 = pow(c.m_e_eV, 2.0);
    kp.r_gamref = 1.0 / kp.gamref;
    kp.r_betaref = 1.0 / kp.betaref;
    kp.r_pref = 1.0 / kp.pref;
    kp.r_grbr = 1.0 / kp.grbr;
    kp.r_m2 = 1.0 / kp.m2;
    kp.four_pi_eps0 = 4 * c.pi * c.epsilon_0;
    kp.phi_norm = 1.0 / ((double)kp.Mx * (double)kp.My * (double)kp.Mz);
    kp.gamref_f = (float)kp.gamref;
    kp.betaref_f = (float)kp.betaref;
    kp.grbr_f = (float)kp.grbr;
    kp.pref_f = (float)kp.pref;
    kp.ipref_f = (float)(1.0 / kp.pref);
    kp.m_f = (float)kp.m_e_eV;
    kp.m2_f = kp.m_f * kp.m_f;
    kp.igrbr2_f = (float)(1.0 / (kp.grbr * kp.grbr));
    for (int k = 0; k < 3; ++k) kp.wait_limit[k] = p.wait_limit[k];
    return kp;
}

extern "C" {

int sc_abi_version(void) { return SC_ABI_VERSION; }

const char* sc_last_error(void) { return g_err.c_str(); }

int sc_plan_create(sc_plan** out, int nx, int ny, int nz, int mode) {
    const int precision = mode & 0x0f;
    if (!out) return fail(SC_ERR_ARG, "plan pointer is NULL");
    *out = nullptr;
    if (nx < 4 || ny < 4 || nz < 4)
        return fail(SC_ERR_ARG, "nmesh_xyz=[%d,%d,%d]: every mesh dimension must be >= 4", nx, ny, nz);
    if (precision != SC_FP64 && precision != SC_FP32) return fail(SC_ERR_ARG, "unknown precision %d", precision);
    if (mode & ~(0x0f | SC_FP32_SORTED_DEPOSIT | SC_FP32_EXACT_IGF | SC_FP32_SPECTRAL_FIELDS))
        return fail(SC_ERR_ARG, "unknown mode bits 0x%x", mode);
    Plan p;
    memset(&p, 0, sizeof p);
    p.nx = nx; p.ny = ny; p.nz = nz;
    p.prec = precision;
    p.sorted_deposit = precision == SC_FP64 || (mode & SC_FP32_SORTED_DEPOSIT);
    p.exact_igf = precision == SC_FP64 || (mode & SC_FP32_EXACT_IGF);
    p.spectral = precision == SC_FP32 && (mode & SC_FP32_SPECTRAL_FIELDS);
    p.Mx = choose_fft_length(nx);
    p.My = choose_fft_length(ny);
    p.Mz = choose_fft_length(nz);
    if (!p.Mx || !p.My || !p.Mz)
        return fail(SC_ERR_UNSUPPORTED, "nmesh_xyz=[%d,%d,%d]: each dimension must be <= 256", nx, ny, nz);
    if (!make_radix_plan(p.Mx, &p.rx) || !make_radix_plan(p.My, &p.ry) || !make_radix_plan(p.Mz, &p.rz))
        return fail(SC_ERR_UNSUPPORTED, "no radix plan");
    const uint64_t ncell = (uint64_t)nx * ny * nz;
    int bits = 0;
    while ((1ull << bits) < ncell) ++bits;
    p.key_bits = bits;
    int dev = 0;
    SC_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    SC_CUDA(cudaDeviceGetAttribute(&p.sm_count, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    p.part_blocks = p.sm_count * 4;
    for (int k = 0; k < 3; ++k) p.wait_limit[k] = MBAR_WAIT_LIMIT;
    p.kick_variant = default_kick_variant();
    p.fft_plane_fwd = p.fft_plane_inv = 1;
    p.fft_cols_x = p.fft_cols_y = 0;
    // everything that is not a stream operation happens here, so that kicks
    // can be recorded in a CUDA graph
    SC_CUDA(prepare_fft_kernels(p), "kernel attributes");
    SC_CUDA(prepare_green_kernels(p), "kernel attributes");
    SC_CUDA(prepare_particle_kernels(), "kernel attributes");
    sc_plan* h = new (std::nothrow) sc_plan;
    if (!h) return fail(SC_ERR_OOM, "out of host memory");
    h->p = p;
    h->ws_ready = nullptr;
    h->ws_ready_bytes = 0;
    h->profiling = false;
    h->last_launches = 0;
    for (int i = 0; i < NEV; ++i) h->ev[i] = nullptr;
    h->side = nullptr;
    h->fork = h->join = nullptr;
    h->status_host = nullptr;
    // the Green's-function branch runs at the highest priority: its FP64
    // blocks take their SM slots first and the keys kernel fills the rest.
    // On any failure sc_plan_destroy releases what was created so far.
    int prio_lo = 0, prio_hi = 0;
    const char* where = "cudaDeviceGetStreamPriorityRange";
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (!e) where = "cudaStreamCreate", e = cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, prio_hi);
    if (!e) where = "cudaEventCreate", e = cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming);
    if (!e) where = "cudaEventCreate", e = cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming);
    if (!e) where = "cudaMallocHost", e = cudaMallocHost(reinterpret_cast<void**>(&h->status_host), sizeof(int));
    if (e) {
        sc_plan_destroy(h);
        return cuda_fail(e, where);
    }
    *out = h;
    return SC_OK;
}

void sc_plan_destroy(sc_plan* plan) {
    if (!plan) return;
    if (plan->profiling)
        for (int i = 0; i < NEV; ++i) cudaEventDestroy(plan->ev[i]);
    if (plan->side) {
        cudaStreamSynchronize(plan->side);
        cudaStreamDestroy(plan->side);
    }
    if (plan->fork) cudaEventDestroy(plan->fork);
    if (plan->join) cudaEventDestroy(plan->join);
    if (plan->status_host) cudaFreeHost(plan->status_host);
    delete plan;
}

int sc_profile_enable(sc_plan* plan, int enable) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (enable && !plan->profiling) {
        for (int i = 0; i < NEV; ++i) {
            const cudaError_t e = cudaEventCreate(&plan->ev[i]);
            if (e) {
                for (int j = 0; j < i; ++j) cudaEventDestroy(plan->ev[j]);
                for (int j = 0; j < NEV; ++j) plan->ev[j] = nullptr;
                return cuda_fail(e, "cudaEventCreate");
            }
        }
        plan->profiling = true;
    } else if (!enable && plan->profiling) {
        for (int i = 0; i < NEV; ++i) cudaEventDestroy(plan->ev[i]);
        plan->profiling = false;
    }
    return SC_OK;
}

int sc_profile_read(sc_plan* plan, float* ms, int* n_launches) {
    if (!plan || !ms) return fail(SC_ERR_ARG, "bad arguments");
    if (!plan->profiling) return fail(SC_ERR_ARG, "profiling is not enabled");
    SC_CUDA(cudaEventSynchronize(plan->ev[9]), "cudaEventSynchronize");
    // main-stream stages, then the two side-stream stages; the convolution is
    // its forward passes (5 -> 13, before the join) plus the rest (6 -> 7),
    // the join wait is 13 -> 6
    static const int a[SC_NSTAGES] = {0, 1, 2, 3, 4, 10, 11, 13, 6, 7, 8};
    static const int b[SC_NSTAGES] = {1, 2, 3, 4, 5, 11, 12, 6, 7, 8, 9};
    for (int i = 0; i < SC_NSTAGES; ++i) SC_CUDA(cudaEventElapsedTime(&ms[i], plan->ev[a[i]], plan->ev[b[i]]), "cudaEventElapsedTime");
    float fwd = 0.f;
    SC_CUDA(cudaEventElapsedTime(&fwd, plan->ev[5], plan->ev[13]), "cudaEventElapsedTime");
    ms[8] += fwd;
    if (n_launches) *n_launches = plan->last_launches;
    return SC_OK;
}

int sc_kick_launches(const sc_plan* plan) { return plan ? plan->last_launches : 0; }

int sc_plan_set_param(sc_plan* plan, int param, int value) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    switch (param) {
        case SC_PARAM_KICK_VARIANT:
            if (value < 0 || value >= SC_KICK_NVARIANTS)
                return fail(SC_ERR_ARG, "kick variant %d not in [0, %d)", value, SC_KICK_NVARIANTS);
            plan->p.kick_variant = value;
            return SC_OK;
        case SC_PARAM_RECORD_FIELD:
            if (value != 0 && value != 1) return fail(SC_ERR_ARG, "record field must be 0 or 1");
            plan->p.record_field = value;
            return SC_OK;
        case SC_PARAM_FFT_PLANE_FWD:
        case SC_PARAM_FFT_PLANE_INV:
            if (value != 0 && value != 1) return fail(SC_ERR_ARG, "FFT plane parameter must be 0 or 1");
            (param == SC_PARAM_FFT_PLANE_FWD ? plan->p.fft_plane_fwd : plan->p.fft_plane_inv) = value;
            return SC_OK;
        case SC_PARAM_FFT_COLS_X:
        case SC_PARAM_FFT_COLS_Y:
            if (value != 0 && value != 2 && value != 4 && value != 8 && value != 16)
                return fail(SC_ERR_ARG, "FFT columns per block must be 0, 2, 4, 8 or 16");
            (param == SC_PARAM_FFT_COLS_X ? plan->p.fft_cols_x : plan->p.fft_cols_y) = value;
            return SC_OK;
        default: return fail(SC_ERR_ARG, "unknown plan parameter %d", param);
    }
}

int sc_plan_get_param(const sc_plan* plan, int param, int* value) {
    if (!plan || !value) return fail(SC_ERR_ARG, "plan or value is NULL");
    switch (param) {
        case SC_PARAM_KICK_VARIANT: *value = plan->p.kick_variant; return SC_OK;
        case SC_PARAM_RECORD_FIELD: *value = plan->p.record_field; return SC_OK;
        case SC_PARAM_FFT_PLANE_FWD: *value = plan->p.fft_plane_fwd; return SC_OK;
        case SC_PARAM_FFT_PLANE_INV: *value = plan->p.fft_plane_inv; return SC_OK;
        case SC_PARAM_FFT_COLS_X: *value = plan->p.fft_cols_x; return SC_OK;
        case SC_PARAM_FFT_COLS_Y: *value = plan->p.fft_cols_y; return SC_OK;
        default: return fail(SC_ERR_ARG, "unknown plan parameter %d", param);
    }
}

int sc_kick_variant(int variant, int* tile, int* stages, int* particles_per_thread, int* blocks_per_sm) {
    int t = 0, st = 0, ppt = 0, mb = 0;
    if (!kick_variant_info(variant, &t, &st, &ppt, &mb))
        return fail(SC_ERR_ARG, "kick variant %d not in [0, %d)", variant, SC_KICK_NVARIANTS);
    if (tile) *tile = t;
    if (stages) *stages = st;
    if (particles_per_thread) *particles_per_thread = ppt;
    if (blocks_per_sm) *blocks_per_sm = mb;
    return SC_OK;
}

int sc_plan_set_wait_limit(sc_plan* plan, int kernel, long long tries) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (kernel < -1 || kernel > 2) return fail(SC_ERR_ARG, "kernel %d: SC_WAIT_FRAME, _EXTENT, _KICK or -1", kernel);
    const unsigned lim = tries < 0 ? MBAR_WAIT_LIMIT : (tries > (long long)MBAR_WAIT_LIMIT ? MBAR_WAIT_LIMIT
                                                                                        : (unsigned)tries);
    for (int k = 0; k < 3; ++k)
        if (kernel < 0 || kernel == k) plan->p.wait_limit[k] = lim;
    return SC_OK;
}

const char* sc_profile_stage_name(int stage) {
    return (stage >= 0 && stage < SC_NSTAGES) ? kStageNames[stage] : "";
}

int sc_plan_fft_shape(const sc_plan* plan, int* mx, int* my, int* mz) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (mx) *mx = plan->p.Mx;
    if (my) *my = plan->p.My;
    if (mz) *mz = plan->p.Mz;
    return SC_OK;
}

int64_t sc_workspace_bytes(const sc_plan* plan, int64_t n_max) {
    if (!plan || n_max < 0) return -1;
    return (int64_t)make_layout(plan->p, n_max).total;
}

int sc_workspace_region(const sc_plan* plan, int64_t n_max, int region, int64_t* offset, int64_t* bytes) {
    if (!plan || !offset || !bytes || n_max < 0) return fail(SC_ERR_ARG, "bad arguments");
    const Layout L = make_layout(plan->p, n_max);
    const size_t rs = plan->p.prec == SC_FP64 ? 8 : 4;
    const size_t ncell = (size_t)plan->p.nx * plan->p.ny * plan->p.nz;
    switch (region) {
        case SC_REGION_QGRID: *offset = (int64_t)L.qgrid; *bytes = (int64_t)(rs * ncell); break;
        case SC_REGION_PHI: *offset = (int64_t)L.phi; *bytes = (int64_t)(rs * ncell); break;
        case SC_REGION_EX: *offset = (int64_t)L.ex; *bytes = (int64_t)(rs * ncell); break;
        case SC_REGION_EY: *offset = (int64_t)L.ey; *bytes = (int64_t)(rs * ncell); break;
        case SC_REGION_EZ: *offset = (int64_t)L.ez; *bytes = (int64_t)(rs * ncell); break;
        case SC_REGION_KEYS: *offset = (int64_t)L.keys; *bytes = (int64_t)(4 * (size_t)n_max); break;
        case SC_REGION_FIELD:
            *offset = (int64_t)L.X;
            *bytes = (int64_t)(rs * 3 * (size_t)((n_max + 3) / 4 * 4));
            break;
        case SC_REGION_STATUS:
            *offset = (int64_t)(L.state + offsetof(ScState, status));
            *bytes = (int64_t)sizeof(int);
            break;
        case SC_REGION_FIRST_ERROR:
            *offset = (int64_t)(L.state + offsetof(ScState, first_error));
            *bytes = (int64_t)sizeof(int);
            break;
        case SC_REGION_IGF: *offset = (int64_t)L.igf_k1; *bytes = (int64_t)(rs * ncell); break;
        default: return fail(SC_ERR_ARG, "unknown region %d", region);
    }
    return SC_OK;
}

int sc_workspace_init(const sc_plan* plan_c, void* ws, size_t ws_bytes, void* stream) {
    sc_plan* plan = const_cast<sc_plan*>(plan_c);
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (!ws) return fail(SC_ERR_WORKSPACE, "workspace is NULL");
    const Layout L = make_layout(plan->p, 0);
    if (ws_bytes < L.total) return fail(SC_ERR_WORKSPACE, "workspace smaller than the fixed part (%zu bytes)", L.total);
    SC_CUDA(launch_init_workspace(plan->p, L, static_cast<char*>(ws), (cudaStream_t)stream), "init workspace");
    plan->ws_ready = ws;
    plan->ws_ready_bytes = ws_bytes;
    return SC_OK;
}

int sc_read_status(const sc_plan* plan, void* ws, void* stream) {
    if (!plan || !ws) return fail(SC_ERR_ARG, "plan or workspace is NULL");
    const Layout L = make_layout(plan->p, 0);
    // one wait for the stream: the status word follows the work already queued
    // on it (copies of the results included) into pinned memory
    SC_CUDA(cudaMemcpyAsync(plan->status_host, static_cast<char*>(ws) + L.state + offsetof(ScState, status),
                            sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream),
            "read status");
    SC_CUDA(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
    const int status = *plan->status_host;
    if (status == SC_ERR_DEGENERATE)
        return fail(status, "degenerate beam: zero or non-finite extent or total charge (mesh step would be 0)");
    if (status == SC_ERR_NONFINITE)
        return fail(status, "non-finite particle coordinates or momenta (or a particle outside the mesh)");
    if (status == SC_ERR_TIMEOUT)
        return fail(status, "a device-side wait for a bulk copy gave up after its iteration limit");
    if (status) return fail(status, "device status %d", status);
    return SC_OK;
}

int sc_kick(sc_plan* plan, void* ws_v, size_t ws_bytes, double* rp, int64_t ld, const double* q, int64_t n,
            double energy_gev, double zstep, double mesh_scale, double mesh_shift, void* stream) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (zstep == 0) return SC_OK;  // sc.py:210-212
    if (n < 1) return fail(SC_ERR_ARG, "n=%lld: the kick needs at least one particle", (long long)n);
    if (n > 0x7fffffffLL) return fail(SC_ERR_ARG, "n=%lld exceeds 2^31-1", (long long)n);
    if (!rp || !q) return fail(SC_ERR_ARG, "rparticles or q is NULL");
    if (ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    if (!(energy_gev > 0) || !isfinite(energy_gev) || !isfinite(zstep))
        return fail(SC_ERR_ARG, "energy %g GeV / zstep %g invalid", energy_gev, zstep);
    const PhysConst c = phys_const();
    if (!(energy_gev / c.m_e_GeV > 1.0)) return fail(SC_ERR_ARG, "energy %g GeV is below the rest mass", energy_gev);
    int r = check_ws(plan, ws_v, ws_bytes, n);
    if (r) return r;
    const Plan& p = plan->p;
    const Layout L = make_layout(p, n);
    char* ws = static_cast<char*>(ws_v);
    cudaStream_t s = (cudaStream_t)stream;
    const KickParams kp = make_params(p, n, ld, energy_gev, zstep, mesh_scale, mesh_shift);
    const int passes = sort_passes(p.key_bits);
    cudaStream_t side = plan->side;
    mark(plan, 0, s);
    SC_CUDA(launch_frame(p, L, ws, kp, rp, s), "frame");
    mark(plan, 1, s);
    SC_CUDA(launch_extent(p, L, ws, kp, rp, q, s), "extent");
    mark(plan, 2, s);
    // fork: the FP64 Green's-function table and its spectrum (they need only
    // the mesh step) run on the side stream while the deposit runs here
    SC_CUDA(cudaEventRecord(plan->fork, s), "cudaEventRecord");
    SC_CUDA(cudaStreamWaitEvent(side, plan->fork, 0), "cudaStreamWaitEvent");
    mark(plan, 10, side);
    SC_CUDA(launch_igf(p, L, ws, side), "igf");
    mark(plan, 11, side);
    SC_CUDA(launch_green_spectrum(p, L, ws, side), "green spectrum");
    mark(plan, 12, side);
    SC_CUDA(cudaEventRecord(plan->join, side), "cudaEventRecord");
    // keys; in the FP32 form the exact fixed-point deposit rides along
    SC_CUDA(launch_keys(p, L, ws, kp, rp, p.sorted_deposit ? nullptr : q, s, p.prec == SC_FP32), "keys");
    mark(plan, 3, s);
    if (p.sorted_deposit) {
        SC_CUDA(launch_sort(reinterpret_cast<uint32_t*>(ws + L.keys), n, p.key_bits, reinterpret_cast<uint32_t*>(ws + L.sort_keys),
                            reinterpret_cast<uint32_t*>(ws + L.sort_perm), reinterpret_cast<uint32_t*>(ws + L.sort_tmp_k),
                            reinterpret_cast<uint32_t*>(ws + L.sort_tmp_v), reinterpret_cast<uint32_t*>(ws + L.sort_hist),
                            reinterpret_cast<uint32_t*>(ws + L.sort_tot), s, q, ws + L.sort_q, p.prec == SC_FP32),
                "sort");
        mark(plan, 4, s);
        SC_CUDA(launch_deposit(p, L, ws, q, n, s), "deposit");
    } else {
        mark(plan, 4, s);
    }
    mark(plan, 5, s);
    // the z and y forward passes need only the charge grid: they run before
    // the join, beside the Green's-function build
    const long long* qfix = p.sorted_deposit ? nullptr : reinterpret_cast<const long long*>(ws + L.qfix);
    SC_CUDA(launch_convolve(p, L, ws, ws + L.qgrid, ws + L.phi, s, qfix, CONV_FORWARD), "convolve");
    mark(plan, 13, s);
    SC_CUDA(cudaStreamWaitEvent(s, plan->join, 0), "cudaStreamWaitEvent");  // join
    mark(plan, 6, s);
    // the kick's field octs do not read the potential: with spectral fields it
    // is produced only for the record-field mode
    SC_CUDA(launch_convolve(p, L, ws, ws + L.qgrid, ws + L.phi, s, qfix, CONV_REST, true, p.record_field != 0),
            "convolve");
    mark(plan, 7, s);
    SC_CUDA(launch_field_grids(p, L, ws, s), "field grids");
    mark(plan, 8, s);
    SC_CUDA(launch_gather_kick(p, L, ws, kp, rp, s), "gather/kick");
    mark(plan, 9, s);
    // frame 1, extent 1, keys 1, [sort 3 per pass, deposit 2], igf 2, green 3, convolve 3 (plane passes) or 5,
    // field 1, kick 1
    plan->last_launches = 1 + 1 + 1 + (p.sorted_deposit ? 3 * passes + 2 : 0) + 2 + 3 + convolve_launches(p) + 1 + 1;
    return SC_OK;
}

int sc_el_field(sc_plan* plan, void* ws_v, size_t ws_bytes, double* X, const double* q, int64_t n, double gamma,
                double mesh_scale, double mesh_shift, double* exyz, void* stream) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (n < 1) return fail(SC_ERR_ARG, "n=%lld: el_field needs at least one particle", (long long)n);
    if (!X || !q || !exyz) return fail(SC_ERR_ARG, "NULL buffer");
    if (!(gamma >= 1.0)) return fail(SC_ERR_ARG, "gamma %g < 1", gamma);
    int r = check_ws(plan, ws_v, ws_bytes, n);
    if (r) return r;
    const Plan& p = plan->p;
    const Layout L = make_layout(p, n);
    char* ws = static_cast<char*>(ws_v);
    cudaStream_t s = (cudaStream_t)stream;
    const KickParams kp = make_params(p, n, n, 1.0, 1.0, mesh_scale, mesh_shift);
    SC_CUDA(launch_extent_xyz(p, L, ws, kp, X, q, gamma, s), "extent");
    SC_CUDA(launch_keys(p, L, ws, kp, nullptr, p.sorted_deposit ? nullptr : q, s), "keys");
    if (p.sorted_deposit) {
        SC_CUDA(launch_sort(reinterpret_cast<uint32_t*>(ws + L.keys), n, p.key_bits, reinterpret_cast<uint32_t*>(ws + L.sort_keys),
                            reinterpret_cast<uint32_t*>(ws + L.sort_perm), reinterpret_cast<uint32_t*>(ws + L.sort_tmp_k),
                            reinterpret_cast<uint32_t*>(ws + L.sort_tmp_v), reinterpret_cast<uint32_t*>(ws + L.sort_hist),
                            reinterpret_cast<uint32_t*>(ws + L.sort_tot), s, q, ws + L.sort_q, p.prec == SC_FP32),
                "sort");
        SC_CUDA(launch_deposit(p, L, ws, q, n, s), "deposit");
    }
    SC_CUDA(launch_igf(p, L, ws, s), "igf");
    SC_CUDA(launch_green_spectrum(p, L, ws, s), "green spectrum");
    SC_CUDA(launch_convolve(p, L, ws, ws + L.qgrid, ws + L.phi, s,
                            p.sorted_deposit ? nullptr : reinterpret_cast<const long long*>(ws + L.qfix), CONV_ALL, true),
            "convolve");
    SC_CUDA(launch_field_grids(p, L, ws, s), "field grids");
    SC_CUDA(launch_gather_xyz(p, L, ws, kp, exyz, s), "gather");
    return SC_OK;
}

int sc_potential(sc_plan* plan, void* ws_v, size_t ws_bytes, const double* qgrid, double hx, double hy, double hz,
                 double* phi, void* stream) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (!qgrid || !phi) return fail(SC_ERR_ARG, "NULL buffer");
    if (!(hx > 0 && hy > 0 && hz > 0) || !isfinite(hx * hy * hz)) return fail(SC_ERR_ARG, "mesh steps must be > 0");
    int r = check_ws(plan, ws_v, ws_bytes, 0);
    if (r) return r;
    const Plan& p = plan->p;
    const Layout L = make_layout(p, 0);
    char* ws = static_cast<char*>(ws_v);
    cudaStream_t s = (cudaStream_t)stream;
    const KickParams kp = make_params(p, 0, 0, 1.0, 1.0, NAN, NAN);
    SC_CUDA(launch_set_mesh(p, L, ws, kp, hx, hy, hz, s), "set mesh");
    SC_CUDA(launch_igf(p, L, ws, s), "igf");
    SC_CUDA(launch_green_spectrum(p, L, ws, s), "green spectrum");
    if (p.prec == SC_FP64) {
        SC_CUDA(launch_convolve(p, L, ws, qgrid, phi, s), "convolve");
    } else {
        const size_t ncell = (size_t)p.nx * p.ny * p.nz;
        launch(k_convert<double, float>, p.sm_count * 4, 256, 0, s, qgrid, reinterpret_cast<float*>(ws + L.qgrid), ncell);
        SC_CUDA(launch_convolve(p, L, ws, ws + L.qgrid, ws + L.phi, s), "convolve");
        launch(k_convert<float, double>, p.sm_count * 4, 256, 0, s, reinterpret_cast<float*>(ws + L.phi), phi, ncell);
        SC_CUDA(cudaGetLastError(), "convert");
    }
    return SC_OK;
}

int sc_sym_kernel(sc_plan* plan, void* ws_v, size_t ws_bytes, double hx, double hy, double hz, double* kern,
                  void* stream) {
    if (!plan) return fail(SC_ERR_ARG, "plan is NULL");
    if (!kern) return fail(SC_ERR_ARG, "NULL buffer");
    int r = check_ws(plan, ws_v, ws_bytes, 0);
    if (r) return r;
    const Layout L = make_layout(plan->p, 0);
    SC_CUDA(launch_igf_h(plan->p, L, static_cast<char*>(ws_v), kern, hx, hy, hz, (cudaStream_t)stream), "igf");
    return SC_OK;
}

int64_t sc_sort_workspace_bytes(int64_t n, int key_bits) {
    if (n < 0 || key_bits < 0 || key_bits > 32) return -1;
    return (int64_t)sort_scratch_bytes(n, key_bits);
}

int sc_sort_keys(const uint32_t* keys_in, int64_t n, int key_bits, uint32_t* keys_out, uint32_t* perm_out, void* ws,
                 size_t ws_bytes, void* stream) {
    if (n < 0 || n > 0x7fffffffLL) return fail(SC_ERR_ARG, "n=%lld out of range", (long long)n);
    if (key_bits < 1 || key_bits > 32) return fail(SC_ERR_ARG, "key_bits=%d not in [1,32]", key_bits);
    if (n == 0) return SC_OK;
    if (!keys_in || !keys_out || !perm_out) return fail(SC_ERR_ARG, "NULL buffer");
    if (keys_in == keys_out) return fail(SC_ERR_ARG, "keys_in must not alias keys_out");
    const size_t need = sort_scratch_bytes(n, key_bits);
    if (!ws || ws_bytes < need) return fail(SC_ERR_WORKSPACE, "sort workspace needs %zu bytes", need);
    char* w = static_cast<char*>(ws);
    const size_t a = align_up(4 * (size_t)n);
    const size_t nb = (size_t)sort_blocks(n);
    uint32_t* tk = reinterpret_cast<uint32_t*>(w);
    uint32_t* tv = reinterpret_cast<uint32_t*>(w + a);
    uint32_t* hist = reinterpret_cast<uint32_t*>(w + 2 * a);
    uint32_t* tot = reinterpret_cast<uint32_t*>(w + 2 * a + align_up(512 * nb * 4));
    SC_CUDA(launch_sort(keys_in, n, key_bits, keys_out, perm_out, tk, tv, hist, tot, (cudaStream_t)stream), "sort");
    return SC_OK;
}

int sc_tmap_apply(const double* R, const double* B, double* rp, int64_t ld, int64_t n, void* stream) {
    if (!R || !B) return fail(SC_ERR_ARG, "R or B is NULL");
    if (n < 0) return fail(SC_ERR_ARG, "n < 0");
    if (n == 0) return SC_OK;
    if (!rp) return fail(SC_ERR_ARG, "rparticles is NULL");
    if (ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    SC_CUDA(launch_tmap(R, B, rp, ld, n, (cudaStream_t)stream), "tmap");
    return SC_OK;
}

// what sc_batch_set saw of a kicked beam's workspace: a kick of the table
// checks it again, so that a workspace initialised anew since (a grown
// workspace, the old one freed) fails instead of being written
struct BatchWs {
    const sc_plan* plan;  // NULL for a transport-only beam
    const void* ws;
    size_t ws_bytes;
    int index;            // the beam's index in the caller's array
};

struct sc_batch {
    int max_beams;
    BatchWs* ws_seen;        // [max_beams], host
    char* h_buf;             // pinned: BatchBeam[max_beams], then int start[BS_COUNT][max_beams + 1]
    char* d_buf;             // device copy
    size_t beams_bytes, start_bytes;
    cudaEvent_t uploaded;    // the last upload's copy has read h_buf
    bool upload_pending;
    int nb;
    int blocks[BS_COUNT];
    size_t fft_smem[3], green_smem[3];
    cudaStream_t side;
    cudaEvent_t fork, join;
    int last_launches;
    bool profiling;
    bool captured;           // a stream capture has recorded this batch's launches
    cudaEvent_t ev[NEV];     // as a plan's: main stream 0..9, side stream 10..13
};

// A kick or transport recorded in a CUDA graph fixes the batch's launch shape
// (see sc_batch_set).
static int note_capture(sc_batch* b, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SC_CUDA(cudaStreamIsCapturing(s, &cs), "cudaStreamIsCapturing");
    if (cs != cudaStreamCaptureStatusNone) b->captured = true;
    return SC_OK;
}

int sc_batch_create(sc_batch** out, int max_beams) {
    if (!out) return fail(SC_ERR_ARG, "batch pointer is NULL");
    *out = nullptr;
    if (max_beams < 1 || max_beams > (1 << 20)) return fail(SC_ERR_ARG, "max_beams=%d out of range", max_beams);
    SC_CUDA(prepare_batch_fft(), "kernel attributes");
    SC_CUDA(prepare_batch_green(), "kernel attributes");
    SC_CUDA(prepare_particle_kernels(), "kernel attributes");
    sc_batch* b = new (std::nothrow) sc_batch;
    if (!b) return fail(SC_ERR_OOM, "out of host memory");
    memset(b, 0, sizeof *b);
    b->max_beams = max_beams;
    b->ws_seen = new (std::nothrow) BatchWs[max_beams];
    if (!b->ws_seen) {
        delete b;
        return fail(SC_ERR_OOM, "out of host memory");
    }
    b->beams_bytes = align_up(sizeof(BatchBeam) * (size_t)max_beams);
    b->start_bytes = sizeof(int) * (size_t)BS_COUNT * (max_beams + 1);
    cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&b->h_buf), b->beams_bytes + b->start_bytes);
    if (!e) e = cudaMalloc(reinterpret_cast<void**>(&b->d_buf), b->beams_bytes + b->start_bytes);
    if (!e) e = cudaEventCreateWithFlags(&b->uploaded, cudaEventDisableTiming);
    int prio_lo = 0, prio_hi = 0;
    if (!e) e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (!e) e = cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, prio_hi);
    if (!e) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
    if (e) {
        sc_batch_destroy(b);
        return cuda_fail(e, "sc_batch_create");
    }
    *out = b;
    return SC_OK;
}

void sc_batch_destroy(sc_batch* b) {
    if (!b) return;
    if (b->profiling)
        for (int i = 0; i < NEV; ++i) cudaEventDestroy(b->ev[i]);
    if (b->side) {
        cudaStreamSynchronize(b->side);
        cudaStreamDestroy(b->side);
    }
    if (b->uploaded) cudaEventSynchronize(b->uploaded), cudaEventDestroy(b->uploaded);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    if (b->d_buf) cudaFree(b->d_buf);
    if (b->h_buf) cudaFreeHost(b->h_buf);
    delete[] b->ws_seen;
    delete b;
}

int sc_batch_set(sc_batch* b, const sc_beam* beams, int nbeams, void* stream) {
    if (!b) return fail(SC_ERR_ARG, "batch is NULL");
    if (nbeams < 0 || nbeams > b->max_beams)
        return fail(SC_ERR_ARG, "nbeams=%d outside [0, %d]", nbeams, b->max_beams);
    if (nbeams && !beams) return fail(SC_ERR_ARG, "beams is NULL");
    const PhysConst c = phys_const();
    // validate everything before touching the table
    std::unordered_map<const void*, int> seen;
    for (int i = 0; i < nbeams; ++i) {
        const sc_beam& m = beams[i];
        if (!m.plan) return fail(SC_ERR_ARG, "beam %d: plan is NULL", i);
        if (m.plan->p.prec != SC_FP32 || m.plan->p.sorted_deposit)
            return fail(SC_ERR_UNSUPPORTED, "beam %d: batched kicks need SC_FP32 plans with the fixed-point deposit", i);
        if (m.zstep == 0 && !m.tmap) continue;  // nothing to do for this beam
        if (m.n < 1 || m.n > 0x7fffffffLL) return fail(SC_ERR_ARG, "beam %d: n=%lld", i, (long long)m.n);
        if (!m.rparticles || !m.q) return fail(SC_ERR_ARG, "beam %d: rparticles or q is NULL", i);
        if (m.ld < m.n) return fail(SC_ERR_ARG, "beam %d: ld=%lld < n=%lld", i, (long long)m.ld, (long long)m.n);
        if (m.zstep == 0) {  // transport only: no kick, so no workspace or energy is used
            if (!seen.emplace((const void*)m.rparticles, i).second)
                return fail(SC_ERR_ARG, "beam %d shares a particle array with beam %d", i, seen[m.rparticles]);
            continue;
        }
        if (!(m.energy_gev > 0) || !isfinite(m.energy_gev) || !isfinite(m.zstep) ||
            !(m.energy_gev / c.m_e_GeV > 1.0))
            return fail(SC_ERR_ARG, "beam %d: energy %g GeV / zstep %g invalid", i, m.energy_gev, m.zstep);
        int r = check_ws(m.plan, m.ws, m.ws_bytes, m.n);
        if (r) return fail(r, "beam %d: %s", i, g_err.c_str());
        for (const void* ptr : {(const void*)m.ws, (const void*)m.rparticles}) {
            if (!seen.emplace(ptr, i).second)
                return fail(SC_ERR_ARG, "beam %d shares a workspace or particle array with beam %d", i, seen[ptr]);
        }
    }
    if (b->upload_pending) SC_CUDA(cudaEventSynchronize(b->uploaded), "cudaEventSynchronize");
    BatchBeam* hb = reinterpret_cast<BatchBeam*>(b->h_buf);
    int* hs = reinterpret_cast<int*>(b->h_buf + b->beams_bytes);
    const int stride = b->max_beams + 1;
    // the new table's launch shape goes into locals: the batch keeps its
    // current table and shape until every check below has passed
    int nb = 0;
    int blocks[BS_COUNT];
    size_t fsm[3] = {0, 0, 0}, gsm[3] = {0, 0, 0};
    std::vector<BatchWs> wsv;
    wsv.reserve(nbeams);
    for (int i = 0; i < nbeams; ++i) {
        const sc_beam& m = beams[i];
        if (m.zstep == 0 && !m.tmap) continue;
        BatchBeam& B = hb[nb];
        memset(&B, 0, sizeof B);
        wsv.push_back(BatchWs{m.zstep == 0 ? nullptr : m.plan, m.ws, m.ws_bytes, i});
        const Plan& p = m.plan->p;
        B.rp = m.rparticles;
        B.q = m.q;
        B.p = p;
        B.gx[BS_TMAP] = batch_particle_blocks(p, m.n);
        B.gy[BS_TMAP] = 1;
        B.has_tm = 1;
        for (int k = 0; k < 42 && m.tmap; ++k) B.tm[k] = m.tmap[k];
        if (m.zstep == 0) {
            // the reference applies the transport of a step whose kick has
            // zero length and skips only the kick (sc.py:210-212): the beam
            // takes part in the transport stage alone, with no blocks in the
            // kick stages
            B.kp.n = m.n;
            B.kp.ld = m.ld;
            ++nb;
            continue;
        }
        B.has_tm = m.tmap != nullptr;
        B.ws = static_cast<char*>(m.ws);
        B.kp = make_params(p, m.n, m.ld, m.energy_gev, m.zstep, m.mesh_scale, m.mesh_shift);
        B.L = make_layout(p, m.n);
        const bool rp_ok = ((uintptr_t)m.rparticles % 16 == 0) && (m.ld % 2 == 0);
        B.vec_rp = rp_ok;
        B.vec_rpq = rp_ok && ((uintptr_t)m.q % 16 == 0);
        size_t fs[3], gs[3];
        batch_fft_tiling(B, fs);
        batch_green_tiling(B, gs);
        for (int k = 0; k < 3; ++k) {
            fsm[k] = fs[k] > fsm[k] ? fs[k] : fsm[k];
            gsm[k] = gs[k] > gsm[k] ? gs[k] : gsm[k];
        }
        B.gx[BS_PART] = batch_particle_blocks(p, m.n);
        B.gy[BS_PART] = 1;
        ++nb;
    }
    for (int st = 0; st < BS_COUNT; ++st) {
        int64_t acc = 0;
        hs[st * stride] = 0;
        for (int i = 0; i < nb; ++i) {
            acc += (int64_t)hb[i].gx[st] * hb[i].gy[st];
            if (acc > 0x7fffffffLL) return fail(SC_ERR_UNSUPPORTED, "batch needs more than 2^31 blocks in a stage");
            hs[st * stride + i + 1] = (int)acc;
        }
        blocks[st] = (int)acc;
    }
    if (b->captured) {
        // a captured graph replays the launches it recorded -- beam count,
        // blocks per stage, dynamic shared memory -- over whatever table is
        // resident: only a table of that shape may replace the current one
        bool same = nb == b->nb;
        for (int st = 0; st < BS_COUNT; ++st) same = same && blocks[st] == b->blocks[st];
        for (int k = 0; k < 3; ++k) same = same && fsm[k] <= b->fft_smem[k] && gsm[k] <= b->green_smem[k];
        if (!same)
            return fail(SC_ERR_ARG,
                        "a CUDA graph recorded this batch's launches for another table shape (number of beams, "
                        "blocks per stage, shared memory): kick these beams with a new batch");
    } else {
        for (int k = 0; k < 3; ++k) b->fft_smem[k] = fsm[k], b->green_smem[k] = gsm[k];
    }
    for (int st = 0; st < BS_COUNT; ++st) b->blocks[st] = blocks[st];
    for (int i = 0; i < nb; ++i) b->ws_seen[i] = wsv[i];
    b->nb = nb;
    cudaStream_t s = (cudaStream_t)stream;
    if (nb) {
        SC_CUDA(cudaMemcpyAsync(b->d_buf, b->h_buf, sizeof(BatchBeam) * nb, cudaMemcpyHostToDevice, s), "upload");
        SC_CUDA(cudaMemcpyAsync(b->d_buf + b->beams_bytes, b->h_buf + b->beams_bytes, b->start_bytes,
                                cudaMemcpyHostToDevice, s),
                "upload");
        SC_CUDA(cudaEventRecord(b->uploaded, s), "cudaEventRecord");
        b->upload_pending = true;
    }
    return SC_OK;
}

static int check_batch_ws(const sc_batch* b) {
    for (int i = 0; i < b->nb; ++i) {
        const BatchWs& w = b->ws_seen[i];
        if (w.plan && (w.plan->ws_ready != w.ws || w.plan->ws_ready_bytes != w.ws_bytes))
            return fail(SC_ERR_WORKSPACE,
                        "beam %d: its plan's workspace was initialised again after sc_batch_set (set the table again)",
                        w.index);
    }
    return SC_OK;
}

int sc_kick_batched(sc_batch* b, void* stream) {
    if (!b) return fail(SC_ERR_ARG, "batch is NULL");
    b->last_launches = 0;
    if (b->nb == 0) return SC_OK;
    if (int r = check_batch_ws(b)) return r;
    cudaStream_t s = (cudaStream_t)stream;
    if (int r = note_capture(b, s)) return r;
    const BatchBeam* beams = reinterpret_cast<const BatchBeam*>(b->d_buf);
    const int* start = reinterpret_cast<const int*>(b->d_buf + b->beams_bytes);
    const int stride = b->max_beams + 1;
    auto row = [&](int st) { return start + st * stride; };
    const int nb = b->nb;
    auto bmark = [&](int i, cudaStream_t st) {
        if (b->profiling) cudaEventRecord(b->ev[i], st);
    };
    bmark(0, s);
    SC_CUDA(launch_batch_particles(BP_FRAME, beams, row(BS_PART), nb, b->blocks[BS_PART], s), "batched frame");
    bmark(1, s);
    SC_CUDA(launch_batch_particles(BP_EXTENT, beams, row(BS_PART), nb, b->blocks[BS_PART], s), "batched extent");
    bmark(2, s);
    SC_CUDA(cudaEventRecord(b->fork, s), "cudaEventRecord");
    SC_CUDA(cudaStreamWaitEvent(b->side, b->fork, 0), "cudaStreamWaitEvent");
    bmark(10, b->side);
    SC_CUDA(launch_batch_igf(beams, row(BS_IGF_C), row(BS_IGF_D), nb, b->blocks[BS_IGF_C], b->blocks[BS_IGF_D],
                             b->side),
            "batched igf");
    bmark(11, b->side);
    const int gb[3] = {b->blocks[BS_GREEN_Z], b->blocks[BS_GREEN_Y], b->blocks[BS_GREEN_X]};
    SC_CUDA(launch_batch_green(beams, row(BS_GREEN_Z), row(BS_GREEN_Y), row(BS_GREEN_X), nb, gb, b->green_smem,
                               b->side),
            "batched green spectrum");
    bmark(12, b->side);
    SC_CUDA(cudaEventRecord(b->join, b->side), "cudaEventRecord");
    SC_CUDA(launch_batch_particles(BP_KEYS, beams, row(BS_PART), nb, b->blocks[BS_PART], s), "batched keys");
    bmark(3, s);
    bmark(4, s);
    bmark(5, s);
    const int fb[5] = {b->blocks[BS_FFT_Z], b->blocks[BS_FFT_Y], b->blocks[BS_FFT_X], b->blocks[BS_FFT_YI],
                       b->blocks[BS_FFT_ZI]};
    SC_CUDA(launch_batch_convolve(beams, row(BS_FFT_Z), row(BS_FFT_Y), row(BS_FFT_X), row(BS_FFT_YI), row(BS_FFT_ZI),
                                  nb, fb, b->fft_smem, s,
                                  CONV_FORWARD),
            "batched convolve");
    bmark(13, s);
    SC_CUDA(cudaStreamWaitEvent(s, b->join, 0), "cudaStreamWaitEvent");
    bmark(6, s);
    SC_CUDA(launch_batch_convolve(beams, row(BS_FFT_Z), row(BS_FFT_Y), row(BS_FFT_X), row(BS_FFT_YI), row(BS_FFT_ZI),
                                  nb, fb, b->fft_smem, s, CONV_REST),
            "batched convolve");
    bmark(7, s);
    SC_CUDA(launch_batch_field(beams, row(BS_FIELD), nb, b->blocks[BS_FIELD], s), "batched field");
    bmark(8, s);
    SC_CUDA(launch_batch_particles(BP_KICK, beams, row(BS_PART), nb, b->blocks[BS_PART], s), "batched kick");
    bmark(9, s);
    // frame, extent, igf 2, green 3, keys, convolve 5, field, kick
    b->last_launches = 1 + 1 + 2 + 3 + 1 + 5 + 1 + 1;
    return SC_OK;
}

int sc_batch_launches(const sc_batch* b) { return b ? b->last_launches : 0; }

int sc_batch_profile_enable(sc_batch* b, int enable) {
    if (!b) return fail(SC_ERR_ARG, "batch is NULL");
    if (enable && !b->profiling) {
        for (int i = 0; i < NEV; ++i) {
            const cudaError_t e = cudaEventCreate(&b->ev[i]);
            if (e) {
                for (int j = 0; j < i; ++j) cudaEventDestroy(b->ev[j]);
                return cuda_fail(e, "cudaEventCreate");
            }
        }
        b->profiling = true;
    } else if (!enable && b->profiling) {
        for (int i = 0; i < NEV; ++i) cudaEventDestroy(b->ev[i]);
        b->profiling = false;
    }
    return SC_OK;
}

int sc_batch_profile_read(sc_batch* b, float* ms) {
    if (!b || !ms) return fail(SC_ERR_ARG, "bad arguments");
    if (!b->profiling) return fail(SC_ERR_ARG, "profiling is not enabled");
    SC_CUDA(cudaEventSynchronize(b->ev[9]), "cudaEventSynchronize");
    static const int a[SC_NSTAGES] = {0, 1, 2, 3, 4, 10, 11, 13, 6, 7, 8};
    static const int e[SC_NSTAGES] = {1, 2, 3, 4, 5, 11, 12, 6, 7, 8, 9};
    for (int i = 0; i < SC_NSTAGES; ++i) SC_CUDA(cudaEventElapsedTime(&ms[i], b->ev[a[i]], b->ev[e[i]]), "cudaEventElapsedTime");
    float fwd = 0.f;
    SC_CUDA(cudaEventElapsedTime(&fwd, b->ev[5], b->ev[13]), "cudaEventElapsedTime");
    ms[8] += fwd;
    return SC_OK;
}

int sc_tmap_batched(sc_batch* b, void* stream) {
    if (!b) return fail(SC_ERR_ARG, "batch is NULL");
    if (b->nb == 0) return SC_OK;
    if (int r = note_capture(b, (cudaStream_t)stream)) return r;
    const BatchBeam* beams = reinterpret_cast<const BatchBeam*>(b->d_buf);
    const int* start = reinterpret_cast<const int*>(b->d_buf + b->beams_bytes);
    SC_CUDA(launch_batch_tmap(beams, start + BS_TMAP * (b->max_beams + 1), b->nb, b->blocks[BS_TMAP],
                              (cudaStream_t)stream),
            "batched transfer map");
    return SC_OK;
}

int sc_tmap_apply_indexed(const double* table, int* counter, int nmaps, double* rp, int64_t ld, int64_t n,
                          void* stream) {
    if (!table || !counter) return fail(SC_ERR_ARG, "table or counter is NULL");
    if (nmaps < 1 || n < 0) return fail(SC_ERR_ARG, "nmaps < 1 or n < 0");
    if (n == 0) return SC_OK;
    if (!rp) return fail(SC_ERR_ARG, "rparticles is NULL");
    if (ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    SC_CUDA(launch_tmap_indexed(table, counter, nmaps, rp, ld, n, (cudaStream_t)stream), "tmap");
    return SC_OK;
}

int sc_tmap2_apply(const double* maps, int nmaps, double* rp, int64_t ld, int64_t n, void* stream) {
    static_assert(SC_MAP2_DOUBLES == 36 + 6 + 6 * 21, "second-order map layout");
    if (nmaps < 0 || n < 0) return fail(SC_ERR_ARG, "nmaps < 0 or n < 0");
    if (nmaps == 0 || n == 0) return SC_OK;
    if (!maps || !rp) return fail(SC_ERR_ARG, "maps or rparticles is NULL");
    if (ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    SC_CUDA(launch_tmap2(maps, nullptr, nmaps, rp, ld, n, (cudaStream_t)stream), "tmap2");
    return SC_OK;
}

int sc_tmap2_apply_step(const double* maps, const int* first, int* counter, int nsteps, double* rp, int64_t ld,
                        int64_t n, void* stream) {
    if (!maps || !first || !counter) return fail(SC_ERR_ARG, "maps, first or counter is NULL");
    if (nsteps < 1 || n < 0) return fail(SC_ERR_ARG, "nsteps < 1 or n < 0");
    if (n > 0 && !rp) return fail(SC_ERR_ARG, "rparticles is NULL");
    if (n > 0 && ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    SC_CUDA(launch_tmap2_step(maps, nullptr, first, counter, nsteps, rp, ld, n, (cudaStream_t)stream), "tmap2");
    return SC_OK;
}

int64_t sc_moments_scratch_bytes(void) { return (int64_t)moments_scratch_bytes(); }

int sc_moments(const double* rp, int64_t ld, int64_t n, const int* counter, int nslots, int use_bounds, double lo,
               double hi, double* out, void* scratch, void* stream) {
    if (!out || !scratch) return fail(SC_ERR_ARG, "out or scratch is NULL");
    if (n < 1 || nslots < 1) return fail(SC_ERR_ARG, "n < 1 or nslots < 1");
    if (!rp) return fail(SC_ERR_ARG, "rparticles is NULL");
    if (ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    if (use_bounds && !(lo <= hi)) return fail(SC_ERR_ARG, "bounds: lo must be <= hi");
    SC_CUDA(launch_moments(rp, ld, n, counter, nslots, use_bounds ? 1 : 0, lo, hi, out, scratch,
                           (cudaStream_t)stream), "moments");
    return SC_OK;
}

int sc_slices_apply(const double* maps, const int* kinds, int nmaps, double* rp, int64_t ld, int64_t n,
                    void* stream) {
    if (nmaps < 0 || n < 0) return fail(SC_ERR_ARG, "nmaps < 0 or n < 0");
    if (nmaps == 0 || n == 0) return SC_OK;
    if (!maps || !kinds || !rp) return fail(SC_ERR_ARG, "maps, kinds or rparticles is NULL");
    if (ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    SC_CUDA(launch_tmap2(maps, kinds, nmaps, rp, ld, n, (cudaStream_t)stream), "slices");
    return SC_OK;
}

int sc_slices_apply_step(const double* maps, const int* kinds, const int* first, int* counter, int nsteps,
                         double* rp, int64_t ld, int64_t n, void* stream) {
    if (!maps || !kinds || !first || !counter) return fail(SC_ERR_ARG, "maps, kinds, first or counter is NULL");
    if (nsteps < 1 || n < 0) return fail(SC_ERR_ARG, "nsteps < 1 or n < 0");
    if (n > 0 && !rp) return fail(SC_ERR_ARG, "rparticles is NULL");
    if (n > 0 && ld < n) return fail(SC_ERR_ARG, "row stride ld=%lld < n=%lld", (long long)ld, (long long)n);
    SC_CUDA(launch_tmap2_step(maps, kinds, first, counter, nsteps, rp, ld, n, (cudaStream_t)stream), "slices");
    return SC_OK;
}

}  // extern "C"
