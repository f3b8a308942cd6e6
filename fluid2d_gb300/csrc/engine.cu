// engine.cu -- device-resident multigrid and model time steppers.
//
//   Gmg    : core/gmg/hierarchy.py (Gridinfo, set_msk_laplacian, Vcycle,
//            Fcycle, solve, twoVcycle) on one GPU, one rank.
//   Model  : core/euler.py, core/boussinesq.py, core/quasigeostrophic.py
//            stepped with core/timescheme.py:167-180 (RK3_SSP), the
//            Operators of core/operators.py and the set_dt of
//            core/fluid2d.py:376-397, all on the device: a step makes no
//            host synchronisation, so it can be captured in a CUDA graph.
//
// Set-up reuses the drop-in kernels (restrict, fillhalo, coarsenmatrix) to
// build every level's mask and Galerkin operator on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <mutex>
#include <vector>

#include "../../include/fluid2d_gb300.h"
#include "f2d_common.cuh"
#include "f2d_fused.cuh"
#include "f2d_kernels.cuh"
#include "f2d_adv.cuh"
#include "f2d_mixed.cuh"
#include "f2d_loop.cuh"
#include "f2d_flux.cuh"
#include "f2d_walls.cuh"
#include "f2d_batch.cuh"
#include <string>

namespace f2d {

int batch_create(int n, int (*step_fn)(void *ctx, int i), void *ctx, int policy, void **out);
int batch_step(void *b, int nsteps, cudaStream_t s);
int batch_info(void *b, int *launches, int *ops);
void batch_destroy(void *b);

#define TRY(x)                      \
    do {                            \
        int _st = (x);              \
        if (_st) return _st;        \
    } while (0)

// ------------------------------------------------------------ arena
// One cudaMalloc per object; sub-buffers 256-byte aligned.
struct Arena {
    std::vector<size_t> sizes;
    char *base = nullptr;
    size_t total = 0;
    size_t add(size_t bytes) {
        size_t o = total;
        total += (bytes + 255) & ~(size_t)255;
        sizes.push_back(bytes);
        return o;
    }
    int alloc() {
        if (total == 0) total = 256;
        TRY(cuda_status(cudaMalloc((void **)&base, total), "engine cudaMalloc"));
        return cuda_status(cudaMemset(base, 0, total), "engine cudaMemset");
    }
    template <typename P>
    P *at(size_t o) const { return (P *)(base + o); }
    ~Arena() {
        if (base) cudaFree(base);
    }
};

// ------------------------------------------------------------ setup kernels
// A0 (9 planes) = stencil*coef*msk(nb)*msk on rows/cols 1..m-2
// (core/gmg/level.py:281-298); the halo is filled afterwards.
__global__ void k_a0_9(const int8_t *msk, int mv, int nv, const double *sc9, double *A9) {
    int i = 1 + blockIdx.x * 32 + threadIdx.x;
    int j = 1 + blockIdx.y * 8 + threadIdx.y;
    if (i > nv - 2 || j > mv - 2) return;
    const size_t pl = (size_t)mv * nv;
    for (int k = 0; k < 9; k++) {
        int di = k % 3 - 1, dj = k / 3 - 1;
        A9[k * pl + off(j, i, nv)] =
            sc9[k] * (double)msk[off(j + dj, i + di, nv)] * (double)msk[off(j, i, nv)];
    }
}

__global__ void k_fill_value(double *x, size_t n, double v) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        x[q] = v;
}

__global__ void k_i8_to_f64(const int8_t *m, double *x, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        x[q] = (double)m[q];
}

// coarse mask: ones, zero where the restricted fine mask <= 0.5 (core/gmg/level.py:233-236)
__global__ void k_threshold(const double *coef, int8_t *msk, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        msk[q] = coef[q] <= 0.5 ? 0 : 1;
}

// keep planes 0..4, Helmholtz shift of A5 (core/gmg/hierarchy.py:80-84),
// C3 = omega/|A5|, plus float copies for the mixed form
__global__ void k_finalize_A(const double *A9, int qg, double rd2inv, double omega, double *A6,
                             float *A6f, size_t pl) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < pl;
         q += (size_t)gridDim.x * blockDim.x) {
        double a[5];
        for (int k = 0; k < 5; k++) a[k] = A9[k * pl + q];
        if (qg && a[4] != 0.) a[4] -= rd2inv;
        for (int k = 0; k < 5; k++) A6[k * pl + q] = a[k];
        double c3 = omega / fabs(a[4]);
        A6[5 * pl + q] = c3;
        if (A6f) {
            for (int k = 0; k < 5; k++) A6f[k * pl + q] = (float)a[k];
            A6f[5 * pl + q] = (float)c3;
        }
    }
}

static int blocks_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)(b > 4096 ? 4096 : (b ? b : 1));
}

// ------------------------------------------------------------ solve control
struct SolveState {
    double normb, res0, res;
    int nite, ndiv, active, status, maxite;
    double tol;
};

// after the first residual: normb, res0, active (core/gmg/hierarchy.py:158-169)
struct SolveInitArgs {
    SolveState *st;
    const double *sumb, *sumr;
    int maxite;
    double tol;
};

F2D_DEV void solve_init_body(const SolveInitArgs &a, const VB) {
    SolveState *st = a.st;
    const double *sumb = a.sumb, *sumr = a.sumr;
    const int maxite = a.maxite;
    const double tol = a.tol;
    double normb = sqrt(sumb[0] / 1.0);
    st->normb = normb;
    st->nite = 0;
    st->ndiv = 0;
    st->status = 0;
    st->maxite = maxite;
    st->tol = tol;
    if (normb > 0) {
        st->res0 = sqrt(sumr[0] / 1.0) / normb;
        st->res = st->res0;
        st->active = (0 < maxite) && (st->res0 > tol);
    } else {
        st->res0 = 0.;
        st->res = 0.;
        st->active = 0;
    }
}

__global__ void k_solve_init(SolveInitArgs a) { pdl_prologue();
    solve_init_body(a, F2D_VB_NATIVE); }

struct BSolveInit {
    using Args = SolveInitArgs;
    static constexpr int THREADS = 1, KIND = BK_SolveInit;
    F2D_DEV static void run(const Args &a, VB vb) { solve_init_body(a, vb); }
};
F2D_BATCH_ENTRY(SolveInit, BSolveInit)

static int solve_init(SolveState *st, const double *sumb, const double *sumr, int maxite,
                      double tol, cudaStream_t s) {
    return launch_body<BSolveInit>(k_solve_init, SolveInitArgs{st, sumb, sumr, maxite, tol},
                                   dim3(1), dim3(1), 0, s, "solve init");
}

// after each F-cycle's residual (core/gmg/hierarchy.py:172-188)
struct SolveUpdateArgs {
    SolveState *st;
    const double *sumr;
};

F2D_DEV void solve_update_body(const SolveUpdateArgs &a, const VB) {
    SolveState *st = a.st;
    const double *sumr = a.sumr;
    if (!st->active) return;
    double res = sqrt(sumr[0] / 1.0) / st->normb;
    double conv = st->res0 / res;
    st->res0 = res;
    st->res = res;
    st->nite += 1;
    if (conv < 1) st->ndiv += 1;
    if (st->ndiv > 4) {
        st->status = ERR_DIVERGED;
        st->active = 0;
        return;
    }
    st->active = (st->nite < st->maxite) && (st->res0 > st->tol);
}

__global__ void k_solve_update(SolveUpdateArgs a) { pdl_prologue();
    solve_update_body(a, F2D_VB_NATIVE); }

struct BSolveUpdate {
    using Args = SolveUpdateArgs;
    static constexpr int THREADS = 1, KIND = BK_SolveUpdate;
    F2D_DEV static void run(const Args &a, VB vb) { solve_update_body(a, vb); }
};
F2D_BATCH_ENTRY(SolveUpdate, BSolveUpdate)

static int solve_update(SolveState *st, const double *sumr, cudaStream_t s) {
    return launch_body<BSolveUpdate>(k_solve_update, SolveUpdateArgs{st, sumr}, dim3(1), dim3(1),
                                     0, s, "solve update");
}

// ------------------------------------------------------------ Gmg
struct LevelInfo {
    int n, m;       // interior
    double dx, dy;
};

// core/gmg/level.py:24-117 for one rank, stopping before an odd dimension
static std::vector<LevelInfo> gridinfo(int n, int m, double dx, double dy, int n0 = 4) {
    std::vector<LevelInfo> v;
    for (int lev = 0;; lev++) {
        if (lev > 0) {
            n /= 2;
            m /= 2;
            dx *= 2;
            dy *= 2;
        }
        bool last = (n <= n0) || (m <= n0) || (n % 2 == 1) || (m % 2 == 1);
        v.push_back({n, m, dx, dy});
        if (last || lev >= MAX_LEVELS - 1) break;
    }
    return v;
}

// ---- L2 persisting windows
// 1 (default): the multigrid cycles' launches carry a persisting L2
// access-policy window over the hierarchy's small levels (and the coarse
// operator's application over the operator), so that the finest level's
// streaming does not evict them between visits; 0: none
static int &l2_persist_mode() {
    static int m = 1;
    return m;
}

// bytes of L2 set aside for persisting accesses in this process's context
// (a context limit, released with the context): the device's maximum, at
// most 32 MB; 0 if unavailable
static size_t l2_setaside() {
    static long long bytes = -1;
    if (bytes < 0) {
        bytes = 0;
        int dev = 0, maxb = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&maxb, cudaDevAttrMaxPersistingL2CacheSize, dev) == cudaSuccess &&
            maxb > 0) {
            const size_t want = std::min<size_t>((size_t)maxb, (size_t)32 << 20);
            if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) == cudaSuccess)
                bytes = (long long)want;
        }
        (void)cudaGetLastError();
    }
    return (size_t)bytes;
}

// a persisting window over [p, p + bytes) (hit ratio scaled to the set-aside)
static cudaAccessPolicyWindow l2_persist_window(void *p, size_t bytes) {
    cudaAccessPolicyWindow w = {};
    const size_t aside = l2_setaside();
    int dev = 0, maxw = 0;
    if (!aside || !p || !bytes || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess ||
        maxw <= 0) {
        (void)cudaGetLastError();
        return w;
    }
    w.base_ptr = p;
    w.num_bytes = std::min(bytes, (size_t)maxw);
    w.hitRatio = (float)std::min(1.0, (double)aside / (double)w.num_bytes);
    w.hitProp = cudaAccessPropertyPersisting;
    w.missProp = cudaAccessPropertyStreaming;
    return w;
}

// the window `w` on this thread's launches for the guard's lifetime (not
// while a step is being recorded: a merged launch serves many instances)
struct L2Guard {
    cudaAccessPolicyWindow prev = {};
    bool on;
    explicit L2Guard(const cudaAccessPolicyWindow &w)
        : on(w.num_bytes > 0 && l2_persist_mode() && recorder() == nullptr) {
        if (on) {
            prev = l2_window();
            l2_window() = w;
        }
    }
    ~L2Guard() {
        if (on) l2_window() = prev;
    }
};

struct Gmg {
    int nlev = 0;
    std::vector<LevelInfo> info;
    int mv[MAX_LEVELS], nv[MAX_LEVELS];
    double omega = 8. / 9.;
    int ndeepest = 16;
    Analytic an{};
    AnalyticT<float> anf{};
    template <typename T>
    const AnalyticT<T> *analytic() const;
    int cs = 1;      // first level of the coarse CTA (== nlev: none)
    int cs_min = 1;  // the finest level whose suffix fits the CTA's shared memory
    size_t smem64 = 0, smem32 = 0;
    Arena mem;
    LevelView<double> d[MAX_LEVELS];
    LevelView<float> f[MAX_LEVELS];
    bool has_f32 = false;
    double *work = nullptr;      // reduction workspace (RED_MAX_BLOCKS * RED_MAX_VALUES)
    double *sums = nullptr;      // 4 device scalars
    SolveState *solve_state = nullptr;
    double *x0_extra = nullptr;  // level-0 correction for solve (the reference's self.x[0])
    // optional timing probe: CUDA events around every finest-level smooth
    // (the two sweep kernels) recorded on the launching stream
    static constexpr int MAX_PROBES = 64;
    bool probe = false;
    int nprobe = 0;
    cudaEvent_t ev[MAX_PROBES][2] = {};
    // The coarse part from level cs started from x = 0 as dense linear maps
    // of the level's interior b (product build): [0] the V-cycle, [1] the
    // F-cycle, for op_n <= COARSE_OP_MAX interior points.
    static constexpr int COARSE_OP_MAX = 1024;
    bool coarse_op = true;
    int op_cs = -1, op_n = 0;
    double *opd[2] = {};
    float *opf[2] = {};
    template <typename T>
    const T *op(int k) const;
    int build_coarse_op(cudaStream_t s);
    // the mixed form's cluster sub-cycle (product build): from float level
    // cl_lev (-1: none) down to the operator's level op_cs
    int cl_lev = -1;
    size_t cl_smem = 0;
    ClArgs cl_tmpl = {};
    void cluster_setup();
    bool cluster_from(int l1, int stop) const {
        return cl_lev >= 0 && cl_lev >= l1 && cl_lev < stop && op_cs == cs && cluster_mode() &&
               recorder() == nullptr;
    }
    int cluster_cycle(LevelView<float> *L, int mode, const int *active, cudaStream_t s) {
        ClArgs a = cl_tmpl;
        a.x_top = L[cl_lev].x;
        a.b_top = L[cl_lev].b;
        a.op = opf[mode == CYCLE_F ? 1 : 0];
        a.op_v = opf[0];
        a.mode = mode;
        a.active = active;
        return mg_cluster_cycle(a, cl_smem, s);
    }
    void free_coarse_op() {
        for (int k = 0; k < 2; k++) {
            if (opd[k]) cudaFree(opd[k]);
            if (opf[k]) cudaFree(opf[k]);
            opd[k] = nullptr;
            opf[k] = nullptr;
        }
        op_cs = -1;
        op_n = 0;
        cl_lev = -1;
        l2w_op[0] = l2w_op[1] = {};
    }
    ~Gmg() {
        for (int k = 0; k < MAX_PROBES; k++)
            for (int e = 0; e < 2; e++)
                if (ev[k][e]) cudaEventDestroy(ev[k][e]);
        free_coarse_op();
    }

    int setup(const int8_t *mskp_host, int nx, int ny, double dx, double dy, double hydroeps,
              double om, bool qg, double Rd, bool f32, cudaStream_t s);
    // level l is smoothed by the fused one-kernel smoother (output into the
    // level's other buffer, the views' x/t pointers swapped afterwards):
    // every level but a float64 finest level, which is FP64-ALU bound and
    // gains nothing from recomputing a ring of first-sweep values
    template <typename T>
    bool fused(int l) const { return !tri && (l > 0 || sizeof(T) == 4); }
    // line relaxation on every level (hydroepsilon*dy/dx <= 0.2,
    // core/gmg/level.py:153-163): elimination factors per level
    bool tri = false;
    double *gam[MAX_LEVELS] = {}, *bet[MAX_LEVELS] = {};
    // levels >= 1 (float64 product build): flags of the points whose stored
    // stencil is the level's uniform one (null: none) and that stencil
    // (c, ey, ex, c3), for the column-form sweeps
    // L2 persisting windows: the small levels' arrays (the cycles' launches)
    // and the coarse operators (their application)
    static constexpr size_t L2_WINDOW_MAX = 24u << 20;
    cudaAccessPolicyWindow l2w_levels = {}, l2w_op[2] = {};
    uint8_t *ufl[MAX_LEVELS] = {};
    double ust[MAX_LEVELS][5] = {};  // (c, ey, ex, c3, a5)
    float ustf[MAX_LEVELS][5] = {};  // the same in float (the float planes are its casts)
    template <typename T>
    const T *uniform_stencil(int l) const;
    template <typename T>
    int smooth(LevelView<T> *L, int l, int xmode, const int *active, cudaStream_t s);
    template <typename T>
    int coarse(LevelView<T> *L, int start, int mode, bool zero_first, const int *active,
               cudaStream_t s);
    template <typename T>
    int vcycle(LevelView<T> *L, int l1, bool zero_first, const int *active, cudaStream_t s,
               int first_mode = 0);
    template <typename T>
    int fcycle(LevelView<T> *L, int l1, const int *active, cudaStream_t s);
};

template <>
const AnalyticT<double> *Gmg::analytic<double>() const { return &an; }
template <>
const AnalyticT<float> *Gmg::analytic<float>() const { return &anf; }
template <>
const double *Gmg::uniform_stencil<double>(int l) const { return ust[l]; }
template <>
const float *Gmg::uniform_stencil<float>(int l) const { return ustf[l]; }
template <>
const double *Gmg::op<double>(int k) const { return opd[k]; }
template <>
const float *Gmg::op<float>(int k) const { return opf[k]; }

template <typename T>
static CoarseArgs<T> coarse_args(const Gmg &g, const LevelView<T> *L, int start, int mode,
                                 bool zero_first, const int *active) {
    CoarseArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.nlev = g.nlev - start;
    for (int l = start; l < g.nlev; l++) a.lev[l - start] = L[l];
    a.c1 = (T)g.omega;
    a.c2 = (T)(1. - g.omega);
    a.mode = mode;
    a.zero_first = zero_first;
    a.ndeepest = g.ndeepest;
    a.active = active;
    return a;
}

// (Re)build the coarse operators for the current cs: column k of each is the
// cycle applied to the unit vector of interior point k, computed by the same
// shared-memory cycle kernel.  The exact build keeps the reference's order of
// operations everywhere and builds none.
int Gmg::build_coarse_op(cudaStream_t s) {
    free_coarse_op();
#ifdef F2D_EXACT
    return OK;
#else
    if (!coarse_op || tri || cs >= nlev) return OK;
    const int m2 = mv[cs] - 2 * NH, n2 = nv[cs] - 2 * NH;
    if (m2 < NH || n2 < NH || (long long)m2 * n2 > COARSE_OP_MAX) return OK;
    const int n = m2 * n2;
    const size_t nn = (size_t)n * n;
    // a hierarchy with float levels (the mixed form) cycles in float; its
    // float64 cycles (the flux diagnostic's) keep the shared-memory CTA
    for (int k = 0; k < 2; k++) {
        if (has_f32)
            TRY(cuda_status(cudaMalloc((void **)&opf[k], nn * sizeof(float)), "coarse operator"));
        else
            TRY(cuda_status(cudaMalloc((void **)&opd[k], nn * sizeof(double)), "coarse operator"));
    }
    const size_t sm64 = coarse_smem_bytes<double>(mv + cs, nv + cs, nlev - cs);
    const size_t sm32 = coarse_smem_bytes<float>(mv + cs, nv + cs, nlev - cs);
    for (int k = 0; k < 2; k++) {
        const int mode = k == 0 ? CYCLE_V : CYCLE_F;
        if (has_f32)
            TRY(mg_coarse_columns<float>(coarse_args<float>(*this, f, cs, mode, true, nullptr),
                                         sm32, opf[k], n, s));
        else
            TRY(mg_coarse_columns<double>(coarse_args<double>(*this, d, cs, mode, true, nullptr),
                                          sm64, opd[k], n, s));
    }
    op_cs = cs;
    op_n = n;
    for (int k = 0; k < 2; k++)
        l2w_op[k] = has_f32 ? l2_persist_window(opf[k], nn * sizeof(float))
                            : l2_persist_window(opd[k], nn * sizeof(double));
    cluster_setup();
    return OK;
#endif
}

// The cluster sub-cycle's layout: the finest float level Ls >= 1, at most
// cluster_mode() levels above the operator's level, whose strips (the
// operator level's interior rows split over CL_NC CTAs, doubled on each
// finer level, CL_G ghost rows a side; x twice, b, t) and the gathered
// coarse b fit in CL_SMEM_MAX bytes a CTA.  None with the switch off,
// without float levels and operator, below CL_NC operator-level rows, or if
// the device cannot hold such a cluster.
void Gmg::cluster_setup() {
    cl_lev = -1;
#ifndef F2D_EXACT
    if (!has_f32 || tri || op_cs < 0 || !opf[0] || !opf[1]) return;
    const int K = op_cs, mc = mv[K] - 2 * NH;
    if (mc < CL_NC) return;
    const int above = cluster_mode();  // levels above the operator's level
    for (int ls = std::max(1, K - above); ls < K; ls++) {
        const int nl = K - ls + 1;
        if (nl > CL_MAXLEV) continue;
        ClArgs a = {};
        a.nlev = nl;
        int strip = 0;
        for (int c = 0; c <= CL_NC; c++) a.p[c] = c * mc / CL_NC;
        for (int c = 0; c < CL_NC; c++) strip = std::max(strip, a.p[c + 1] - a.p[c]);
        size_t o = 0;
        for (int k = 0; k < nl; k++) {
            const int l = ls + k;
            ClLevel &v = a.lv[k];
            v.mv = mv[l];
            v.nv = nv[l];
            v.rows = (strip << (nl - 1 - k)) + 2 * CL_G;
            v.msk = f[l].msk;
            v.A = f[l].A;
            const size_t bytes = ((size_t)v.rows * v.nv * sizeof(float) + 15) & ~(size_t)15;
            v.o_x[0] = (unsigned)o;
            v.o_x[1] = (unsigned)(o + bytes);
            v.o_b = (unsigned)(o + 2 * bytes);
            v.o_t = (unsigned)(o + 3 * bytes);
            o += 4 * bytes;
        }
        a.o_g = (unsigned)o;
        a.n = op_n;
        o += ((size_t)op_n * sizeof(float) + 15) & ~(size_t)15;
        a.c2 = (float)(1. - omega);
        if (o > CL_SMEM_MAX) continue;
        if (!mg_cluster_feasible(o)) return;
        cl_tmpl = a;
        cl_smem = o;
        cl_lev = ls;
        return;
    }
#endif
}

int Gmg::setup(const int8_t *mskp_host, int nx, int ny, double dx, double dy, double hydroeps,
               double om, bool qg, double Rd, bool f32, cudaStream_t s) {
    omega = om;
    info = gridinfo(nx, ny, dx, dy);
    nlev = (int)info.size();
    for (int l = 0; l < nlev; l++) {
        if (info[l].n < NH || info[l].m < NH) {
            set_error("multigrid: level %d is %dx%d, below the halo width", l, info[l].n,
                      info[l].m);
            return ERR_SHAPE;
        }
        nv[l] = info[l].n + 2 * NH;
        mv[l] = info[l].m + 2 * NH;
        const bool t = hydroeps * info[l].dy / info[l].dx <= .2;
        if (l == 0) tri = t;
        if (t != tri) {
            set_error("multigrid: levels with and without the tridiagonal relaxation");
            return ERR_ARG;
        }
    }
    if (tri && f32) {
        set_error("multigrid: the tridiagonal relaxation runs in float64 only");
        return ERR_ARG;
    }
    if (tri && mv[0] > 5632) {
        set_error("multigrid: %d rows exceed the line relaxation's column buffers", mv[0]);
        return ERR_LIMIT;
    }
    has_f32 = f32;
    // first level of the coarse CTA: the largest suffix of levels >= 1 that
    // fits in shared memory
    cs = nlev;
    for (int l = nlev - 1; l >= 1 && !tri; l--) {
        if (coarse_smem_bytes<double>(mv + l, nv + l, nlev - l) <= 200 * 1024) cs = l;
        else break;
    }
    cs_min = cs;
    if (cs < nlev) {
        smem64 = coarse_smem_bytes<double>(mv + cs, nv + cs, nlev - cs);
        smem32 = coarse_smem_bytes<float>(mv + cs, nv + cs, nlev - cs);
    }

    // ---- memory
    size_t o_msk[MAX_LEVELS], o_A[MAX_LEVELS], o_Af[MAX_LEVELS], o_x[MAX_LEVELS],
        o_b[MAX_LEVELS], o_r[MAX_LEVELS], o_t[MAX_LEVELS], o_xf[MAX_LEVELS], o_bf[MAX_LEVELS],
        o_rf[MAX_LEVELS], o_tf[MAX_LEVELS], o_A9[MAX_LEVELS];
    size_t maxpl = 0;
    for (int l = 0; l < nlev; l++) {
        size_t pl = (size_t)mv[l] * nv[l];
        maxpl = pl > maxpl ? pl : maxpl;
        o_msk[l] = mem.add(pl);
        o_A[l] = l > 0 ? mem.add(6 * pl * sizeof(double)) : 0;
        o_Af[l] = (l > 0 && f32) ? mem.add(6 * pl * sizeof(float)) : 0;
        o_x[l] = mem.add(pl * sizeof(double));
        o_b[l] = mem.add(pl * sizeof(double));
        o_r[l] = mem.add(pl * sizeof(double));
        o_t[l] = mem.add(pl * sizeof(double));
        if (f32) {
            o_xf[l] = mem.add(pl * sizeof(float));
            o_bf[l] = mem.add(pl * sizeof(float));
            o_rf[l] = mem.add(pl * sizeof(float));
            o_tf[l] = mem.add(pl * sizeof(float));
        }
    }
    // the arrays the cycles read, level by level, are contiguous: the small
    // levels' span is the L2 persisting window (set-up-only arrays follow)
    const size_t o_levels_end = mem.total;
    for (int l = 0; l < nlev; l++) o_A9[l] = mem.add(9 * (size_t)mv[l] * nv[l] * sizeof(double));
    size_t o_coef = mem.add(maxpl * sizeof(double));
    size_t o_work = mem.add(sizeof(double) * RED_MAX_BLOCKS * RED_MAX_VALUES);
    size_t o_sums = mem.add(8 * sizeof(double));
    size_t o_solve = mem.add(sizeof(SolveState));
    size_t o_sc9 = mem.add(16 * sizeof(double));
    size_t o_ones = mem.add(maxpl);
    size_t o_nb = mem.add(sizeof(uint16_t) * (size_t)mv[0] * nv[0]);
    size_t o_gam[MAX_LEVELS] = {}, o_bet[MAX_LEVELS] = {};
    if (tri)
        for (int l = 0; l < nlev; l++) {
            o_gam[l] = mem.add(sizeof(double) * (size_t)mv[l] * nv[l]);
            o_bet[l] = mem.add(sizeof(double) * (size_t)mv[l] * nv[l]);
        }
    size_t o_uf[MAX_LEVELS] = {}, o_smp = 0;
#ifndef F2D_EXACT
    if (!tri) {
        for (int l = 1; l < nlev; l++) o_uf[l] = mem.add((size_t)mv[l] * nv[l]);
        o_smp = mem.add(sizeof(double) * 96 * MAX_LEVELS);
    }
#endif
    TRY(mem.alloc());
    {   // the L2 window: the finest level >= 1 from which the levels' arrays fit
        int l2 = 1;
        while (l2 < nlev && o_levels_end - o_msk[l2] > L2_WINDOW_MAX) l2++;
        l2w_levels = {};
        if (l2 < nlev) l2w_levels = l2_persist_window(mem.base + o_msk[l2], o_levels_end - o_msk[l2]);
    }
    work = mem.at<double>(o_work);
    sums = mem.at<double>(o_sums);
    solve_state = mem.at<SolveState>(o_solve);
    for (int l = 0; l < nlev; l++) {
        d[l].mv = f[l].mv = mv[l];
        d[l].nv = f[l].nv = nv[l];
        d[l].msk = f[l].msk = mem.at<int8_t>(o_msk[l]);
        d[l].A = l > 0 ? mem.at<double>(o_A[l]) : nullptr;
        f[l].A = (l > 0 && f32) ? mem.at<float>(o_Af[l]) : nullptr;
        d[l].x = mem.at<double>(o_x[l]);
        d[l].b = mem.at<double>(o_b[l]);
        d[l].r = mem.at<double>(o_r[l]);
        d[l].t = mem.at<double>(o_t[l]);
        d[l].nb = f[l].nb = nullptr;
        if (f32) {
            f[l].x = mem.at<float>(o_xf[l]);
            f[l].b = mem.at<float>(o_bf[l]);
            f[l].r = mem.at<float>(o_rf[l]);
            f[l].t = mem.at<float>(o_tf[l]);
        }
    }
    x0_extra = d[0].x;

    // ---- finest level: mask and analytic operator (core/gmg/level.py:261-302)
    size_t pl0 = (size_t)mv[0] * nv[0];
    TRY(cuda_status(cudaMemcpyAsync((void *)d[0].msk, mskp_host, pl0, cudaMemcpyHostToDevice, s),
                    "mask upload"));
    {  // the analytic operator's coefficient bits, read by every level-0 kernel
        uint16_t *nb = mem.at<uint16_t>(o_nb);
        TRY(mg_nbmask(d[0], nb, s));
        d[0].nb = f[0].nb = nb;
    }
    double bx = dy / dx * hydroeps, by = dx / dy;
    double a = -2 * (bx + by), b = 0., c = 0.;
    double st[9] = {c, by, c, bx, a, bx, c, by, c};
    if (dx == dy && hydroeps == 1) {
        a = -6. / 2;
        b = 1. / 2;
        c = 0.5 / 2;
        double s9[9] = {c, b, c, b, a, b, c, b, c};
        memcpy(st, s9, sizeof(st));
    }
    double coef = 1. / (dx * dy);
    double sc9[9];
    for (int k = 0; k < 9; k++) sc9[k] = st[k] * coef;
    for (int k = 0; k < 5; k++) an.sc[k] = sc9[k];
    an.a5 = sc9[4] * 1. * 1.;
    if (qg) an.a5 -= 1. / (Rd * Rd);
    an.c3 = omega / fabs(an.a5);
    for (int k = 0; k < 5; k++) anf.sc[k] = (float)an.sc[k];
    anf.a5 = (float)an.a5;
    anf.c3 = (float)an.c3;
    TRY(cuda_status(cudaMemcpyAsync(mem.at<double>(o_sc9), sc9, sizeof(sc9),
                                    cudaMemcpyHostToDevice, s),
                    "stencil upload"));
    {
        dim3 bl(32, 8);
        k_a0_9<<<grid2d(mv[0] - 2, nv[0] - 2, bl), bl, 0, s>>>(
            d[0].msk, mv[0], nv[0], mem.at<double>(o_sc9), mem.at<double>(o_A9[0]));
        TRY(launch_status("A0"));
        for (int k = 0; k < 9; k++)
            TRY(launch_fillhalo(mem.at<double>(o_A9[0]) + k * pl0, NH, mv[0], nv[0], s));
    }
    // ---- coarser levels (core/gmg/level.py:227-243, 304-327)
    int8_t *ones = mem.at<int8_t>(o_ones);
    TRY(cuda_status(cudaMemsetAsync(ones, 1, maxpl, s), "ones"));
    double *coefb = mem.at<double>(o_coef);
    double rd2inv = qg ? 1. / (Rd * Rd) : 0.;
    for (int l = 1; l < nlev; l++) {
        size_t plf = (size_t)mv[l - 1] * nv[l - 1], pl = (size_t)mv[l] * nv[l];
        double *mskf = d[l].t;  // scratch: the finer mask as float64 (fits: plf <= 4 pl + ...)
        double *mskf_big = d[l - 1].r;
        (void)mskf;
        k_i8_to_f64<<<blocks_for(plf), 256, 0, s>>>(d[l - 1].msk, mskf_big, plf);
        k_fill_value<<<blocks_for(pl), 256, 0, s>>>(coefb, pl, 1.0);
        TRY(launch_restrict(ones, mskf_big, NH, mv[l], nv[l], mv[l - 1], nv[l - 1], coefb, s));
        TRY(launch_fillhalo(coefb, NH, mv[l], nv[l], s));
        k_threshold<<<blocks_for(pl), 256, 0, s>>>(coefb, (int8_t *)d[l].msk, pl);
        TRY(launch_status("coarse mask"));
        TRY(launch_coarsenmatrix(mem.at<double>(o_A9[l - 1]), d[l - 1].msk, d[l].msk, NH,
                                 mv[l - 1], nv[l - 1], mv[l], nv[l], mem.at<double>(o_A9[l]), s));
        for (int k = 0; k < 9; k++)
            TRY(launch_fillhalo(mem.at<double>(o_A9[l]) + k * pl, NH, mv[l], nv[l], s));
    }
    for (int l = 1; l < nlev; l++) {
        size_t pl = (size_t)mv[l] * nv[l];
        k_finalize_A<<<blocks_for(pl), 256, 0, s>>>(mem.at<double>(o_A9[l]), qg, rd2inv, omega,
                                                    (double *)d[l].A,
                                                    f32 ? (float *)f[l].A : nullptr, pl);
        TRY(launch_status("finalize A"));
    }
#ifndef F2D_EXACT
    // the stored levels' uniform stencils (product build, column-form sweeps)
    if (!tri && nlev > 1) {
        double *smp = mem.at<double>(o_smp);
        for (int l = 1; l < nlev; l++) TRY(mg_stencil_samples(d[l], smp + 96 * l, s));
        double h[96 * MAX_LEVELS];
        TRY(cuda_status(cudaMemcpyAsync(h, smp, sizeof(double) * 96 * nlev,
                                        cudaMemcpyDeviceToHost, s),
                        "stencil samples copy"));
        TRY(cuda_status(cudaStreamSynchronize(s), "stencil samples sync"));
        for (int l = 1; l < nlev; l++) {
            ufl[l] = nullptr;
            if (!mg_uniform_choose(h + 96 * l, ust[l])) continue;
            for (int k = 0; k < 5; k++) ustf[l][k] = (float)ust[l][k];
            ufl[l] = mem.at<uint8_t>(o_uf[l]);
            TRY(mg_uniform_flags(d[l], ust[l], ufl[l], s));
        }
    }
#endif
    for (int l = 0; l < nlev; l++) {
        size_t pl = (size_t)mv[l] * nv[l];
        TRY(cuda_status(cudaMemsetAsync(d[l].r, 0, pl * sizeof(double), s), "clear"));
    }
    if (tri)
        for (int l = 0; l < nlev; l++) {
            gam[l] = mem.at<double>(o_gam[l]);
            bet[l] = mem.at<double>(o_bet[l]);
            TRY(mg_tri_factor(d[l], l == 0 ? &an : nullptr, gam[l], bet[l], s));
        }
    // without its coarse operators (no memory for them) the hierarchy runs
    // the cycle in the coarse CTA: same function, so set-up goes on
    if (build_coarse_op(s) != OK) {
        free_coarse_op();
        (void)cudaGetLastError();
    }
    return OK;
}

template <typename T>
int Gmg::smooth(LevelView<T> *L, int l, int xmode, const int *active, cudaStream_t s) {
    const AnalyticT<T> *a0 = l == 0 ? analytic<T>() : nullptr;
    T c1 = (T)omega, c2 = (T)(1. - omega);
    const bool pr = probe && l == 0 && nprobe < MAX_PROBES;
    if (pr) {
        for (int e = 0; e < 2; e++)
            if (!ev[nprobe][e]) TRY(cuda_status(cudaEventCreate(&ev[nprobe][e]), "probe event"));
        // external record: inside stream capture it becomes an event-record node
        TRY(cuda_status(cudaEventRecordWithFlags(ev[nprobe][0], s, cudaEventRecordExternal),
                        "probe record"));
    }
    if (tri) {
        // Level.smooth with the line relaxation (core/gmg/level.py:340-368):
        // three smoothtridiag sweeps per call, each followed by a halo fill
        if constexpr (sizeof(T) == 8) {
            const size_t n = (size_t)L[l].mv * L[l].nv;
            if (xmode == X_ZERO) TRY(mg_zero(L[l].x, n, active, s));
            if (xmode == X_PLUS_INTERP || xmode == X_INTERP) {
                // coarsetofine writes the whole fine array (nh = 3, no halo
                // fill) and the line relaxation reads its outer columns, so
                // the correction is formed in r and added everywhere
                // (core/gmg/hierarchy.py:118-126, level.py:447-470)
                TRY(launch_interpolate(L[l].msk, L[l + 1].msk, L[l + 1].x, NH, L[l + 1].mv,
                                       L[l + 1].nv, L[l].mv, L[l].nv, L[l].r, s));
                TRY(mg_add(L[l].x, L[l].r, n, xmode == X_INTERP, active, s));
            }
            for (int k = 0; k < 3; k++) {
                TRY(mg_tri_sweep(L[l], l == 0 ? &an : nullptr, gam[l], bet[l], active, s));
                TRY(launch_fillhalo(L[l].x, NH, L[l].mv, L[l].nv, s));
            }
        }
    } else if (fused<T>(l)) {
        // a stored level with a uniform stencil, large enough for the column
        // form (product build): prolongation, then the two sweeps.  The float
        // finest level (mixed form) keeps the fused smoother: its column form
        // measured 19.1 against 17.0 us a call at 1024^2.
        const bool col = l > 0 && ufl[l] != nullptr && column_applies<T>(L[l]);
        if (col) {
            if (xmode == X_PLUS_INTERP || xmode == X_INTERP)
                TRY(mg_interp<T>(L[l + 1], L[l + 1].x, L[l], L[l].x, xmode == X_INTERP, active, s));
            TRY(mg_sweeps_uniform<T>(L[l], ufl[l], uniform_stencil<T>(l), c1, c2, xmode == X_ZERO,
                                     active, s));
        } else {
            TRY(mg_smooth_fused<T>(L[l], a0, c1, c2, xmode,
                                   xmode >= X_PLUS_INTERP ? &L[l + 1] : nullptr, L[l].t, active, s));
            T *tmp = L[l].x;
            L[l].x = L[l].t;
            L[l].t = tmp;
        }
    } else {
        if (xmode == X_PLUS_INTERP || xmode == X_INTERP)
            TRY(mg_interp<T>(L[l + 1], L[l + 1].x, L[l], L[l].x, xmode == X_INTERP, active, s));
        // the column form where it applies (float64 product build), else the
        // sweeps in the reference's order of operations
        bool done = false;
        if constexpr (sizeof(T) == 8)
            if (a0) TRY(mg_sweeps_column<T>(L[l], *a0, c1, c2, xmode == X_ZERO, active, s, &done));
        if (!done) {
            TRY(mg_sweep1<T>(L[l], a0, c1, c2, xmode == X_ZERO, active, s));
            TRY(mg_sweep2<T>(L[l], a0, c1, c2, active, s));
        }
    }
    if (pr) {
        TRY(cuda_status(cudaEventRecordWithFlags(ev[nprobe][1], s, cudaEventRecordExternal),
                        "probe record"));
        nprobe++;
    }
    return OK;
}

template <typename T>
int Gmg::coarse(LevelView<T> *L, int start, int mode, bool zero_first, const int *active,
                cudaStream_t s) {
    if (op_n > 0 && op_cs == cs && start == cs && (mode == CYCLE_F || zero_first)) {
        const T *o = op<T>(mode == CYCLE_F ? 1 : 0);
        L2Guard guard(l2w_op[mode == CYCLE_F ? 1 : 0]);
        if (o) return mg_coarse_apply<T>(o, op_n, L[start], active, s);
    }
    size_t smem = coarse_smem_bytes<T>(mv + start, nv + start, nlev - start);
    return mg_coarse<T>(coarse_args<T>(*this, L, start, mode, zero_first, active), smem, s);
}

// core/gmg/hierarchy.py:98-126.  first_mode: the first level's input is x
// (X_IN) or the prolongation of the next coarser level (X_INTERP, the
// F-cycle's coarsetofine into x followed by this V-cycle).
template <typename T>
int Gmg::vcycle(LevelView<T> *L, int l1, bool zero_first, const int *active, cudaStream_t s,
                int first_mode) {
    L2Guard guard(l2w_levels);
    const int deep = nlev - 1;
    if (l1 >= cs) return coarse(L, l1, CYCLE_V, zero_first, active, s);
    const int stop = cs < deep ? cs : deep;
    // levels [lc, stop) and the coarse part as one cluster launch (float
    // levels, where the first smooth there starts from zero)
    int lc = stop;
    if constexpr (sizeof(T) == 4)
        if (cluster_from(l1, stop) && (zero_first || cl_lev > l1)) lc = cl_lev;
    for (int l = l1; l < lc; l++) {
        const int xm = (zero_first || l > l1) ? X_ZERO : (l == l1 ? first_mode : X_IN);
        TRY(smooth(L, l, xm, active, s));
        const AnalyticT<T> *a0 = l == 0 ? analytic<T>() : nullptr;
        if (fused<T>(l)) {
            TRY(mg_resres<T>(L[l], a0, L[l + 1], L[l + 1].b, active, s, l > 0 ? ufl[l] : nullptr,
                             l > 0 ? uniform_stencil<T>(l) : nullptr));
        } else {
            TRY(mg_residual<T>(L[l], a0, L[l].x, L[l].b, L[l].r, active, s));
            TRY(mg_restrict<T>(L[l], L[l].r, L[l + 1], L[l + 1].b, active, s));
        }
    }
    if (lc < stop) {
        if constexpr (sizeof(T) == 4) TRY(cluster_cycle(L, CYCLE_V, active, s));
    } else if (cs <= deep) {
        TRY(coarse(L, cs, CYCLE_V, true, active, s));
    } else {
        for (int k = 0; k < ndeepest; k++) TRY(smooth(L, deep, k == 0 ? X_ZERO : X_IN, active, s));
    }
    for (int l = lc - 1; l >= l1; l--) TRY(smooth(L, l, X_PLUS_INTERP, active, s));
    return OK;
}

// core/gmg/hierarchy.py:131-151
template <typename T>
int Gmg::fcycle(LevelView<T> *L, int l1, const int *active, cudaStream_t s) {
    L2Guard guard(l2w_levels);
    const int deep = nlev - 1;
    if (l1 >= cs) return coarse(L, l1, CYCLE_F, false, active, s);
    const int stop = cs < deep ? cs : deep;
    int lc = stop;  // levels [lc, stop) and the coarse part as one cluster launch
    if constexpr (sizeof(T) == 4)
        if (cluster_from(l1, stop)) lc = cl_lev;
    for (int l = l1; l < lc; l++) TRY(mg_restrict<T>(L[l], L[l].b, L[l + 1], L[l + 1].b, active, s));
    if (lc < stop) {
        if constexpr (sizeof(T) == 4) TRY(cluster_cycle(L, CYCLE_F, active, s));
    } else if (cs <= deep) {
        TRY(coarse(L, cs, CYCLE_F, false, active, s));
    } else {
        for (int k = 0; k < ndeepest; k++) TRY(smooth(L, deep, k == 0 ? X_ZERO : X_IN, active, s));
    }
    for (int l = lc - 1; l >= l1; l--) TRY(vcycle(L, l, false, active, s, X_INTERP));
    return OK;
}

// twoVcycle (core/gmg/hierarchy.py:207-218): x is updated in place, b read
static int two_vcycle(Gmg &g, double *x, const double *b, cudaStream_t s) {
    LevelView<double> L[MAX_LEVELS];
    for (int l = 0; l < g.nlev; l++) L[l] = g.d[l];
    L[0].x = x;
    L[0].b = (double *)b;
    for (int k = 0; k < 2; k++) TRY(g.vcycle(L, 0, false, nullptr, s));
    return OK;
}

// solve (core/gmg/hierarchy.py:154-192) in correction form, device-resident:
// every iteration is launched; iterations after convergence are no-ops
// through the device flag SolveState::active.
static int solve(Gmg &g, double *x, const double *b, int maxite, double tol, cudaStream_t s) {
    LevelView<double> L[MAX_LEVELS];
    for (int l = 0; l < g.nlev; l++) L[l] = g.d[l];
    LevelView<double> &L0 = L[0];
    // g.residual(x, b, self.b[0])
    TRY(mg_residual<double>(L0, &g.an, x, b, L0.b, nullptr, s));
    TRY(launch_reduce(8, L0.msk, b, nullptr, NH, L0.mv, L0.nv, g.sums + 0, g.work, s));
    TRY(launch_reduce(8, L0.msk, L0.b, nullptr, NH, L0.mv, L0.nv, g.sums + 1, g.work, s));
    TRY(solve_init(g.solve_state, g.sums + 0, g.sums + 1, maxite, tol, s));
    const int *active = &g.solve_state->active;
    const size_t pl = (size_t)L0.mv * L0.nv;
    for (int it = 0; it < maxite; it++) {
        TRY(g.fcycle(L, 0, active, s));
        TRY(vec_add(x, L0.x, pl, active, s));
        TRY(mg_residual<double>(L0, &g.an, x, b, L0.b, active, s));
        TRY(launch_reduce(8, L0.msk, L0.b, nullptr, NH, L0.mv, L0.nv, g.sums + 1, g.work, s));
        TRY(solve_update(g.solve_state, g.sums + 1, s));
    }
    return OK;
}

// ---- mixed form: FP32 cycles inside an FP64 defect correction.
// twoVcycle: x <- x + V32(b - A x), twice.  A V-cycle is linear in its
// right-hand side and initial guess, so V(x, b) = x + V(0, b - A x): in
// exact arithmetic this is the reference's two V-cycles (hierarchy.py:207-218).
static int two_vcycle_mixed(Gmg &g, double *x, const double *b, cudaStream_t s) {
    LevelView<double> L0 = g.d[0];
    LevelView<float> Lf[MAX_LEVELS];
    for (int l = 0; l < g.nlev; l++) Lf[l] = g.f[l];
    const size_t pl = (size_t)L0.mv * L0.nv;
    for (int k = 0; k < 2; k++) {
        TRY(mg_residual_mixed(L0, g.an, x, b, L0.r, Lf[0].b, nullptr, s));
        TRY(g.vcycle(Lf, 0, true, nullptr, s));
        TRY(vec_add_f32(x, Lf[0].x, pl, nullptr, s));
    }
    return OK;
}

// solve (hierarchy.py:154-192) is already in correction form: the F-cycles
// run in FP32 on the FP64 residual, the correction is accumulated in FP64.
static int solve_mixed(Gmg &g, double *x, const double *b, int maxite, double tol,
                       cudaStream_t s) {
    LevelView<double> L0 = g.d[0];
    LevelView<float> Lf[MAX_LEVELS];
    for (int l = 0; l < g.nlev; l++) Lf[l] = g.f[l];
    const size_t pl = (size_t)L0.mv * L0.nv;
    TRY(mg_residual_mixed(L0, g.an, x, b, L0.b, Lf[0].b, nullptr, s));
    TRY(launch_reduce(8, L0.msk, b, nullptr, NH, L0.mv, L0.nv, g.sums + 0, g.work, s));
    TRY(launch_reduce(8, L0.msk, L0.b, nullptr, NH, L0.mv, L0.nv, g.sums + 1, g.work, s));
    TRY(solve_init(g.solve_state, g.sums + 0, g.sums + 1, maxite, tol, s));
    const int *active = &g.solve_state->active;
    for (int it = 0; it < maxite; it++) {
        TRY(g.fcycle(Lf, 0, active, s));
        TRY(vec_add_f32(x, Lf[0].x, pl, active, s));
        TRY(mg_residual_mixed(L0, g.an, x, b, L0.b, Lf[0].b, active, s));
        TRY(launch_reduce(8, L0.msk, L0.b, nullptr, NH, L0.mv, L0.nv, g.sums + 1, g.work, s));
        TRY(solve_update(g.solve_state, g.sums + 1, s));
    }
    return OK;
}

// ------------------------------------------------------------ model
enum ModelKind { M_EULER = 0, M_BOUSSINESQ = 1, M_QG = 2 };

// names of the state variables (core/euler.py:36-37, core/boussinesq.py:30-31,
// core/quasigeostrophic.py:32)
static const char *VARNAMES[3][6] = {
    {"vorticity", "psi", "u", "v", "source", nullptr},
    {"vorticity", "psi", "u", "v", "buoyancy", "banom"},
    {"pv", "psi", "u", "v", "pvanom", "vorticity"}};
static const int NVAR[3] = {5, 6, 6};
__host__ __device__ constexpr int ndiag_of(int kind) { return kind == 2 ? 6 : 8; }
static const int NDIAG[3] = {ndiag_of(0), ndiag_of(1), ndiag_of(2)};
// status word bits (include/fluid2d_gb300.h F2D_STATUS_*)
enum { STATUS_NONFINITE = 1, STATUS_BLOWUP = 2, STATUS_DIVERGED = 4, STATUS_BAD_DT = 8 };

struct DiagArgs {
    int kind;
    const int8_t *msk;
    const double *s;  // state
    size_t pl;
    int mv, nv;
    double dx, dy;     // coordinates xr, yr of core/grid.py:49-52
    double gravity, Rd, area;
    double *part;      // partials
    double *out;       // NDIAG values
    int nr;            // partial kernel: rows per block; final kernel: partial blocks
    int *status;              // the model's status word (F2D_STATUS_* bits, sticky)
    const SolveState *solve;  // the last full solve's state (divergence)
};

// diagnostics of core/euler.py:185-223, core/boussinesq.py:123-153,
// core/quasigeostrophic.py:189-218 in one pass (8 accumulators)
F2D_DEV void diag_partial_body(const DiagArgs &a, const VB blk) {
    __shared__ double sh[8 * RED_THREADS];
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int rpb = a.nr;
    const int rows = a.mv - 2 * NH, cols = a.nv - 2 * NH;
    const int r0 = blk.x * rpb, r1 = min(rows, r0 + rpb);
    const int cells = (r1 - r0) * cols;
    const double *s = a.s;
    const size_t pl = a.pl;
    const int nv = a.nv;
    // thread t takes cells t, t + RED_THREADS, ... in row-major order
    int jr = (int)threadIdx.x / cols, ic = (int)threadIdx.x - jr * cols;
    for (int q = threadIdx.x; q < cells; q += RED_THREADS) {
        const int j = NH + r0 + jr, i = NH + ic;
        ic += RED_THREADS;
        while (ic >= cols) {
            ic -= cols;
            jr++;
        }
        const size_t p = off(j, i, nv);
        const int mc = a.msk[p];
        const double *u = s + 2 * pl, *v = s + 3 * pl;
        if (mc == 1) {  // computekemaxu (core/fortran_diag.f90:179-189)
            double ua = u[p], ub = u[p - 1], va = v[p], vb = v[p - nv];
            acc[1] += (ua * ua + ub * ub) + (va * va + vb * vb);
            double sp = fabs(ua + ub) + fabs(va + vb);
            acc[0] = acc[0] > sp ? acc[0] : sp;
        }
        if (a.kind == M_EULER) {
            const double w = s[p];
            if (mc == 1) {
                acc[2] += w;
                acc[3] += w * w;
            }
            if (mc != 0) {
                double xr = ((double)i + 0.5 - NH + 0) * a.dx;
                double yr = ((double)j + 0.5 - NH + 0) * a.dy;
                acc[4] += w * xr;
                acc[5] += w * yr;
                acc[6] += s[pl + p];          // psi
                acc[7] += w * s[4 * pl + p];  // source
            }
        } else if (a.kind == M_BOUSSINESQ) {
            const double w = s[p], b = s[4 * pl + p];
            if (mc == 1) {
                acc[2] += w;
                acc[3] += w * w;
                acc[5] += b;
                acc[6] += b * b;
            }
            if (mc != 0) {
                double yr = ((double)j + 0.5 - NH + 0) * a.dy;
                acc[4] += b * yr;
            }
        } else {
            const double pv = s[p];
            const double *psi = s + pl;
            if (mc == 1) {
                acc[2] += pv;
                acc[3] += pv * pv;
                // cornertocell (core/fortran_operators.f90:118) then sum of squares
                double wc = 0.25 * (psi[p] + psi[p - 1] + psi[p - nv] + psi[p - nv - 1]);
                acc[4] += wc * wc;
            }
        }
    }
    double v8[8];
    bool mx[8] = {true, false, false, false, false, false, false, false};
    for (int k = 0; k < 8; k++) v8[k] = acc[k];
    block_reduce<8>(v8, mx, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < 8; k++) a.part[k * RED_MAX_BLOCKS + blk.x] = v8[k];
}

__global__ void __launch_bounds__(RED_THREADS) k_diag_partial(DiagArgs a) {
    pdl_prologue();
    diag_partial_body(a, F2D_VB_NATIVE);
}

F2D_DEV void diag_final_body(const DiagArgs &a, const VB) {
    const int nb = a.nr;
    __shared__ double sh[8 * RED_THREADS];
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nb; b += RED_THREADS)
        for (int k = 0; k < 8; k++) {
            double v = a.part[k * RED_MAX_BLOCKS + b];
            acc[k] = k == 0 ? (acc[k] > v ? acc[k] : v) : acc[k] + v;
        }
    bool mx[8] = {true, false, false, false, false, false, false, false};
    block_reduce<8>(acc, mx, sh);
    if (threadIdx.x) return;
    const double area = a.area;
    const double maxu = acc[0] * 0.5, ke = acc[1] * 0.25;
    if (a.kind == M_EULER) {
        a.out[0] = maxu;
        a.out[1] = ke / area;
        a.out[2] = acc[2] / area;
        a.out[3] = 0.5 * acc[3] / area;
        a.out[4] = acc[4] / area;
        a.out[5] = acc[5] / area;
        a.out[6] = acc[6] / area;
        a.out[7] = acc[7] / area;
    } else if (a.kind == M_BOUSSINESQ) {
        const double pe = -a.gravity * acc[4];
        a.out[0] = maxu;
        a.out[1] = ke / area;
        a.out[2] = pe / area;
        a.out[3] = (ke + pe) / area;
        a.out[4] = acc[2] / area;
        a.out[5] = 0.5 * acc[3] / area;
        a.out[6] = acc[5] / area;
        a.out[7] = sqrt(acc[6] / area - (acc[5] / area) * (acc[5] / area));
    } else {
        const double ape = 0.5 * acc[4] / (a.Rd * a.Rd);
        a.out[0] = maxu;
        a.out[1] = ke / area;
        a.out[2] = acc[2] / area;
        a.out[3] = 0.5 * acc[3] / area;
        a.out[4] = ape / area;
        a.out[5] = (ke + ape) / area;
    }
    if (a.status) {
        // what stops the reference's run, per instance: a blow-up
        // (maxspeed > 1e3, core/fluid2d.py:309-314), a diverged solve
        // (core/gmg/hierarchy.py:182-188), and any non-finite value: a NaN or
        // Inf anywhere in u, v or the tracers reaches these sums
        int st = 0;
        bool finite = isfinite(acc[0]) && isfinite(acc[1]);
        for (int k = 0; k < ndiag_of(a.kind); k++) finite = finite && isfinite(a.out[k]);
        if (!finite) st |= STATUS_NONFINITE;
        if (maxu > 1e3) st |= STATUS_BLOWUP;
        if (a.solve && a.solve->status == ERR_DIVERGED) st |= STATUS_DIVERGED;
        if (st) *a.status |= st;
    }
}

__global__ void __launch_bounds__(RED_THREADS) k_diag_final(DiagArgs a) {
    pdl_prologue();
    diag_final_body(a, F2D_VB_NATIVE);
}

struct BDiagP {
    using Args = DiagArgs;
    static constexpr int THREADS = RED_THREADS, KIND = BK_DiagP, MIN_BLOCKS = 4;
    F2D_DEV static void run(const Args &a, VB vb) { diag_partial_body(a, vb); }
};
struct BDiagF {
    using Args = DiagArgs;
    static constexpr int THREADS = RED_THREADS, KIND = BK_DiagF;
    F2D_DEV static void run(const Args &a, VB vb) { diag_final_body(a, vb); }
};
F2D_BATCH_ENTRY(DiagP, BDiagP)
F2D_BATCH_ENTRY(DiagF, BDiagF)

static const char *DIAGNAMES[3][8] = {
    {"maxspeed", "ke", "vorticity", "enstrophy", "px", "py", "angmom", "source"},
    {"maxspeed", "ke", "pe", "energy", "vorticity", "enstrophy", "buoyancy", "brms"},
    {"maxspeed", "ke", "pv", "pv2", "ape", "energy", nullptr, nullptr}};

// set_dt (core/fluid2d.py:376-397): dt and cst[3] = maxspeed of the last
// diagnostics, plus the flux-splitting constants that adv_upwind derives
// from cst (core/fortran_advection.f90:46-60), computed once per step
struct SetDtArgs {
    double *dt, *cst;
    SplitConst *advc;
    const double *diag;
    int adaptable;
    double dt0, cfl, hmin, dtmax;
    int *status;  // STATUS_BAD_DT when the step's dt is not a positive finite number
};

F2D_DEV void set_dt_body(const SetDtArgs &a, const VB) {
    double *dt = a.dt, *cst = a.cst;
    SplitConst *advc = a.advc;
    const double *diag = a.diag;
    const int adaptable = a.adaptable;
    const double dt0 = a.dt0, cfl = a.cfl, hmin = a.hmin, dtmax = a.dtmax;
    const double maxspeed = diag[0];
    double d = dt0;
    if (adaptable && maxspeed != 0) {
        d = cfl * hmin / maxspeed;
        if (d > dtmax) d = dtmax;
    }
    *dt = d;
    cst[3] = maxspeed;
    *advc = split_const(cst);
    if (a.status && !(isfinite(d) && d > 0.)) *a.status |= STATUS_BAD_DT;
}

__global__ void k_set_dt(SetDtArgs a) { pdl_prologue();
    set_dt_body(a, F2D_VB_NATIVE); }

struct BSetDt {
    using Args = SetDtArgs;
    static constexpr int THREADS = 1, KIND = BK_SetDt;
    F2D_DEV static void run(const Args &a, VB vb) { set_dt_body(a, vb); }
};
F2D_BATCH_ENTRY(SetDt, BSetDt)

static int set_dt(double *dt, double *cst, void *advc, const double *diag, int adaptable,
                  double dt0, double cfl, double hmin, double dtmax, int *status,
                  cudaStream_t s) {
    return launch_body<BSetDt>(
        k_set_dt,
        SetDtArgs{dt, cst, (SplitConst *)advc, diag, adaptable, dt0, cfl, hmin, dtmax, status},
        dim3(1), dim3(1), 0, s, "set_dt");
}

// QG fields after the step (core/quasigeostrophic.py:120-122, :186) and the
// Boussinesq anomaly (core/boussinesq.py:99-100)
__global__ void k_qg_post(double *s, size_t pl, const double *pvback, double rdm2, int which) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < pl;
         q += (size_t)gridDim.x * blockDim.x) {
        double pva = s[q] - pvback[q];  // pvanom = pv - pvback
        s[4 * pl + q] = pva;
        if (which) s[5 * pl + q] = pva - rdm2 * s[pl + q];  // vorticity = pvanom - Rd^-2 psi
    }
}

struct BanomArgs {
    double *s;
    size_t pl;
    const double *bref;
};

F2D_DEV void banom_body(const BanomArgs &a, const VB vb) {
    for (size_t q = vb.x * (size_t)blockDim.x + threadIdx.x; q < a.pl;
         q += (size_t)vb.gx * blockDim.x)
        a.s[5 * a.pl + q] = a.s[4 * a.pl + q] - a.bref[q];
}

__global__ void k_banom(BanomArgs a) { pdl_prologue();
    banom_body(a, F2D_VB_NATIVE); }

struct BBanom {
    using Args = BanomArgs;
    static constexpr int THREADS = 256, KIND = BK_Banom;
    F2D_DEV static void run(const Args &a, VB vb) { banom_body(a, vb); }
};
F2D_BATCH_ENTRY(Banom, BBanom)

struct Model {
    f2d_model_desc desc;
    int kind, nvar, mv, nv;
    size_t pl;
    double dx, dy, area;
    Gmg gmg;
    Arena mem;
    int8_t *msk = nullptr, *mskp = nullptr, *ones = nullptr;
    double *X, *D[3], *S1, *S2, *B, *cst, *advc, *dt, *diag, *pvback, *bref, *part;
    int *status = nullptr;  // F2D_STATUS_* bits, set by the diagnostics, sticky
    // mixed form: float stage states, float tendencies, float split constants
    float *Xf = nullptr, *S1f = nullptr, *S2f = nullptr, *Df[3] = {nullptr, nullptr, nullptr};
    float *dtf = nullptr;
    void *advf = nullptr;
    template <typename P>
    P *planef(P *base, const char *name) {
        for (int k = 0; k < nvar; k++)
            if (!strcmp(VARNAMES[kind][k], name)) return base + k * pl;
        return nullptr;
    }
    int stage_mixed(int k, cudaStream_t s);
    // the forcing stage (the third of RK3_SSP) inverts: Boussinesq always,
    // Euler when it diffuses (core/euler.py:156-169)
    bool invert_at_forcing_stage() const {
        return kind == M_BOUSSINESQ || (kind == M_EULER && desc.diffusion);
    }
    // add_diffusion coefficient of tracer t at the forcing stage: Kdiff times
    // the stage coefficient (1; Boussinesq: the RK3_SSP dtcoef 1.5,
    // core/boussinesq.py:106-112), over dx*dx (core/fortran_operators.f90:138)
    double diffusion_coef(int t) const {
        if (!desc.diffusion) return 0.;
        const double K = (kind == M_BOUSSINESQ ? 1.5 : 1.) * desc.Kdiff[t];
        return K / (dx * dx);
    }
    // device time loop (core/fluid2d.py:235-314): clock, rings, WHILE graph
    struct Loop {
        Arena mem;
        LoopClock *clock = nullptr;
        LoopConst k{};
        LoopRings r{};
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaGraphConditionalHandle h = 0;      // WHILE: run another step
        cudaGraphConditionalHandle hflux = 0;  // IF: flux diagnostic this step
        cudaStream_t capture = nullptr;  // private stream the graph is captured on
        ~Loop() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            if (capture) cudaStreamDestroy(capture);
        }
    };
    Loop *loop = nullptr;
    // flux diagnostic (core/fluxes.py:6-213): extended state, its own RK
    // tendencies (persistent, like the reference's Timescheme buffers) and
    // the rev/irr flux planes
    struct Flux {
        Arena mem;
        int ntr = 0, ns = 0, nflx = 0, next = 0, nfull = 0;
        int tr[4] = {0, 0, 0, 0};  // plane of each advected quantity
        double *X = nullptr, *Xe = nullptr, *Xw = nullptr, *S = nullptr, *FLX = nullptr,
               *fcst = nullptr;
        double *D[3] = {nullptr, nullptr, nullptr};
        std::vector<std::string> names;
    };
    Flux *flux = nullptr;
    // no-slip walls (core/operators.py:157-184, 245-290): wall mask, boundary
    // cells, their count, and the source buffer (Euler: the 'source' plane)
    struct Noslip {
        Arena mem;
        int8_t *msk = nullptr, *mskbc = nullptr;
        double *src = nullptr, *sum = nullptr;
        double bcarea = 0.;
    };
    Noslip *noslip = nullptr;
    int noslip_setup(const int8_t *msknoslip_host, cudaStream_t s);
    int add_noslip(cudaStream_t s);
    int flux_setup(cudaStream_t s);
    int flux_rhs(const double *xs, double *dxdt, cudaStream_t s);
    int flux_forward(double sgn, cudaStream_t s);
    int diag_fluxes(cudaStream_t s);
    int loop_body(cudaStream_t s);
    int loop_build(cudaStream_t s);
    int last_nite = 0;
    int probe_per_step = -1;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // the step with the state uploaded from and read back to host memory
    // hptr, captured as one graph (f2d_model_step_host)
    cudaGraph_t hgraph = nullptr;
    cudaGraphExec_t hexec = nullptr;
    double *hptr = nullptr;
    void drop_host_graph() {
        if (hexec) cudaGraphExecDestroy(hexec);
        if (hgraph) cudaGraphDestroy(hgraph);
        hexec = nullptr;
        hgraph = nullptr;
        hptr = nullptr;
    }

    double *plane(double *base, const char *name) {
        for (int k = 0; k < nvar; k++)
            if (!strcmp(VARNAMES[kind][k], name)) return base + k * pl;
        return nullptr;
    }
    int create(const f2d_model_desc *d, const int8_t *msk_host, cudaStream_t s);
    int invert(double *xs, const char *who, bool full, cudaStream_t s, bool island = false);
    // islands with a prescribed streamfunction (core/island.py, core/operators.py:442-444,
    // 482-486): the right-hand-side correction and the psi offset
    struct Islands {
        Arena mem;
        double *rhsp = nullptr, *psi = nullptr;
    };
    Islands *isl = nullptr;
    // psi*mskp (+ the islands' psi) and psi -> (u, v) with the RK options of o
    int ortho(OrthoStage &o, bool island, cudaStream_t s) {
        if (island && isl) {
            TRY(psi_island(o.psi, mskp, isl->psi, pl, s));
            o.premasked = 1;
        }
        return stage_ortho(o, s);
    }
    int stage(int k, cudaStream_t s);
    int step(cudaStream_t s);
    int advance(cudaStream_t s);
    int diagnostics(cudaStream_t s);
    int set_psi(cudaStream_t s);
};

int Model::create(const f2d_model_desc *d, const int8_t *msk_host, cudaStream_t s) {
    desc = *d;
    kind = d->model;
    if (kind < 0 || kind > 2) {
        set_error("model: unknown kind %d", kind);
        return ERR_ARG;
    }
    if (d->nx < 4 || d->ny < 4 || d->nx > (1 << 15) || d->ny > (1 << 15) ||
        !(d->Lx > 0. && d->Ly > 0.) || !isfinite(d->Lx) || !isfinite(d->Ly)) {
        set_error("model: bad grid nx=%d ny=%d Lx=%g Ly=%g", d->nx, d->ny, d->Lx, d->Ly);
        return ERR_SHAPE;
    }
    if (d->order < 1 || d->order > 6 || d->precision < 0 || d->precision > 1 ||
        !(d->dt > 0.) || !isfinite(d->dt)) {
        set_error("model: bad order %d, precision %d or dt %g", d->order, d->precision, d->dt);
        return ERR_ARG;
    }
    nvar = NVAR[kind];
    nv = d->nx + 2 * NH;
    mv = d->ny + 2 * NH;
    pl = (size_t)mv * nv;
    dx = d->Lx / d->nx;
    dy = d->Ly / d->ny;
    // corner mask (core/operators.py:47-67): 1 where the 4 cells around the
    // corner are fluid; the last row and column stay 0 as celltocorner leaves them
    std::vector<int8_t> mp(pl, 0);
    double a = 0.;
    for (int j = 0; j < mv; j++)
        for (int i = 0; i < nv; i++) {
            if (j < mv - 1 && i < nv - 1) {
                double w = 0.25 * ((double)msk_host[off(j, i, nv)] + (double)msk_host[off(j, i + 1, nv)]
                                   + (double)msk_host[off(j + 1, i, nv)]
                                   + (double)msk_host[off(j + 1, i + 1, nv)]);
                mp[off(j, i, nv)] = (w == 1.) ? 1 : 0;
            }
            if (j >= NH && j < mv - NH && i >= NH && i < nv - NH) a += msk_host[off(j, i, nv)];
        }
    area = a * 1.;
    if (area <= 0) {
        set_error("model: the mask has no fluid cell");
        return ERR_ARG;
    }
    size_t o_msk = mem.add(pl), o_mskp = mem.add(pl), o_ones = mem.add(pl);
    size_t o_X = mem.add(nvar * pl * 8), o_D0 = mem.add(nvar * pl * 8),
           o_D1 = mem.add(nvar * pl * 8), o_D2 = mem.add(nvar * pl * 8),
           o_S1 = mem.add(nvar * pl * 8), o_S2 = mem.add(nvar * pl * 8), o_B = mem.add(pl * 8),
           o_cst = mem.add(8 * 8), o_advc = mem.add(sizeof(SplitConst)), o_dt = mem.add(8),
           o_diag = mem.add(8 * 8),
           o_pvb = mem.add(kind == M_QG ? pl * 8 : 8), o_bref = mem.add(kind == M_BOUSSINESQ ? pl * 8 : 8),
           o_part = mem.add(8 * RED_MAX_BLOCKS * 8), o_status = mem.add(16);
    const bool mixed = d->precision != 0;
    size_t o_f[6] = {0, 0, 0, 0, 0, 0}, o_advf = 0, o_dtf = 0;
    if (mixed) {
        for (int k = 0; k < 6; k++) o_f[k] = mem.add(nvar * pl * 4);
        o_advf = mem.add(sizeof(SplitT<float>));
        o_dtf = mem.add(16);
    }
    TRY(mem.alloc());
    if (mixed) {
        Xf = mem.at<float>(o_f[0]);
        S1f = mem.at<float>(o_f[1]);
        S2f = mem.at<float>(o_f[2]);
        for (int k = 0; k < 3; k++) Df[k] = mem.at<float>(o_f[3 + k]);
        advf = mem.at<void>(o_advf);
        dtf = mem.at<float>(o_dtf);
    }
    msk = mem.at<int8_t>(o_msk);
    mskp = mem.at<int8_t>(o_mskp);
    ones = mem.at<int8_t>(o_ones);
    TRY(cuda_status(cudaMemsetAsync(ones, 1, pl, s), "ones"));
    X = mem.at<double>(o_X);
    D[0] = mem.at<double>(o_D0);
    D[1] = mem.at<double>(o_D1);
    D[2] = mem.at<double>(o_D2);
    S1 = mem.at<double>(o_S1);
    S2 = mem.at<double>(o_S2);
    B = mem.at<double>(o_B);
    cst = mem.at<double>(o_cst);
    advc = mem.at<double>(o_advc);
    dt = mem.at<double>(o_dt);
    diag = mem.at<double>(o_diag);
    pvback = mem.at<double>(o_pvb);
    bref = mem.at<double>(o_bref);
    part = mem.at<double>(o_part);
    status = mem.at<int>(o_status);
    TRY(cuda_status(cudaMemsetAsync(status, 0, sizeof(int), s), "status"));
    TRY(cuda_status(cudaMemcpyAsync(msk, msk_host, pl, cudaMemcpyHostToDevice, s), "msk"));
    TRY(cuda_status(cudaMemcpyAsync(mskp, mp.data(), pl, cudaMemcpyHostToDevice, s), "mskp"));
    // cst (core/operators.py:99-119)
    double c[8] = {dx, dy, 0.05, 0., (d->order % 2 == 0) ? 0. : d->aparab, 0, 0, 0};
    TRY(cuda_status(cudaMemcpyAsync(cst, c, sizeof(c), cudaMemcpyHostToDevice, s), "cst"));
    if (kind == M_QG) {
        // pvback = beta*(yr - Ly*0.5)*msk (core/quasigeostrophic.py:50)
        std::vector<double> pb(pl);
        for (int j = 0; j < mv; j++) {
            double yr = ((double)j + 0.5 - NH + 0) * dy;
            for (int i = 0; i < nv; i++)
                pb[off(j, i, nv)] = d->beta * (yr - d->Ly * .5) * (double)msk_host[off(j, i, nv)];
        }
        TRY(cuda_status(cudaMemcpyAsync(pvback, pb.data(), pl * 8, cudaMemcpyHostToDevice, s),
                        "pvback"));
        TRY(cuda_status(cudaStreamSynchronize(s), "pvback sync"));
    }
    TRY(cuda_status(cudaStreamSynchronize(s), "model upload"));
    return gmg.setup(mp.data(), d->nx, d->ny, dx, dy, kind == M_QG ? 1. : d->hydroepsilon, 8. / 9.,
                     kind == M_QG, d->Rd, d->precision != 0, s);
}

// invert_vorticity (core/operators.py:421-498), up to (not including) the
// psi*mskp + orthogradient pass, which the caller fuses with RK updates
int Model::invert(double *xs, const char *who, bool full, cudaStream_t s, bool island) {
    double *w = plane(xs, who), *psi = plane(xs, "psi");
    const bool mixed = desc.precision != 0;
    TRY(launch_celltocorner(w, B, mv, nv, s));
    if (island && isl) TRY(plane_sub(B, isl->rhsp, pl, s));
    if (!full) return mixed ? two_vcycle_mixed(gmg, psi, B, s) : two_vcycle(gmg, psi, B, s);
    if (mixed)
        TRY(solve_mixed(gmg, psi, B, 4, 1e-11, s));
    else
        TRY(solve(gmg, psi, B, 4, 1e-11, s));
    if (desc.perio) {
        // psi -= sum(psi[interior])/area (core/operators.py:474-477), an unmasked sum
        TRY(launch_reduce(2, ones, psi, nullptr, NH, mv, nv, gmg.sums + 2, gmg.work, s));
        TRY(vec_axpy_const(psi, area, gmg.sums + 2, pl, s));
    }
    return OK;
}

static OrthoStage ortho_base(Model &M, double *xs) {
    OrthoStage o;
    memset(&o, 0, sizeof(o));
    o.msk = M.msk;
    o.mskp = M.mskp;
    o.psi = M.plane(xs, "psi");
    o.u = M.plane(xs, "u");
    o.v = M.plane(xs, "v");
    o.zdx = 1. / M.dx;
    o.zdy = 1. / M.dy;
    o.dt = M.dt;
    o.mv = M.mv;
    o.nv = M.nv;
    return o;
}

static AdvStage adv_base(Model &M, const double *xs, const char *tracer, double *dq) {
    AdvStage a;
    memset(&a, 0, sizeof(a));
    a.msk = M.msk;
    a.q = M.plane((double *)xs, tracer);
    a.u = M.plane((double *)xs, "u");
    a.v = M.plane((double *)xs, "v");
    a.advc = M.advc;
    a.dq = M.plane(dq, tracer);
    a.dt = M.dt;
    a.kind = (M.desc.order % 2 == 0) ? 1 : 0;
    a.fp32 = M.desc.precision != 0;
    a.method = M.desc.flux_method;
    a.order = M.desc.order;
    a.mv = M.mv;
    a.nv = M.nv;
    return a;
}

// One RK3_SSP stage k (core/timescheme.py:167-180): rhs(x_k, dx_k) with the
// next stage state (k = 0: S1, k = 1: S2) or the final update (k = 2)
// written by the kernels that produce the tendencies.
int Model::stage(int k, cudaStream_t s) {
    double *xs = k == 0 ? X : (k == 1 ? S1 : S2);
    double *dk = D[k];
    double *out = k == 0 ? S1 : (k == 1 ? S2 : X);
    const int rk = k + 1;
    const char *tracers[2] = {kind == M_QG ? "pv" : "vorticity", "buoyancy"};
    const int ntr = kind == M_BOUSSINESQ ? 2 : 1;
    for (int t = 0; t < ntr; t++) {
        AdvStage a = adv_base(*this, xs, tracers[t], dk);
        if (kind == M_BOUSSINESQ && t == 0) {  // rhs_torque (core/operators.py:303-314)
            a.buoy = plane(xs, "buoyancy");
            a.torque_coef = 0.5 * desc.gravity / dx;
        }
        a.rk = rk;
        a.base = plane(X, tracers[t]);
        a.d0 = k >= 1 ? plane(D[0], tracers[t]) : nullptr;
        a.d1 = k >= 2 ? plane(D[1], tracers[t]) : nullptr;
        a.out = plane(out, tracers[t]);
        if (k == 2) a.diff_coef = diffusion_coef(t);
        TRY(stage_advection(a, s));
    }
    // Euler and QG do not invert at the forcing stage (kforcing = 2,
    // core/euler.py:156-169, core/quasigeostrophic.py:160-168) unless Euler
    // diffuses there; Boussinesq inverts at every stage (core/boussinesq.py:114)
    const bool inv = (kind == M_BOUSSINESQ) || k < 2 || (kind == M_EULER && desc.diffusion);
    if (!inv) return OK;
    if (kind == M_QG) {
        // dxdt[:] = 0 then dxdt[pvanom] = dxdt[pv]: the warm start is zero
        TRY(cuda_status(cudaMemsetAsync(plane(dk, "psi"), 0, pl * 8, s), "qg warm start"));
        TRY(invert(dk, "pv", false, s, true));
    } else {
        TRY(invert(dk, "vorticity", false, s));
    }
    OrthoStage o = ortho_base(*this, dk);
    o.rk = rk;
    o.ubase = plane(X, "u");
    o.vbase = plane(X, "v");
    o.u0 = k >= 1 ? plane(D[0], "u") : nullptr;
    o.v0 = k >= 1 ? plane(D[0], "v") : nullptr;
    o.u1 = k >= 2 ? plane(D[1], "u") : nullptr;
    o.v1 = k >= 2 ? plane(D[1], "v") : nullptr;
    o.uout = plane(out, "u");
    o.vout = plane(out, "v");
    const bool inv2 = invert_at_forcing_stage();
    if (!inv2 && k == 1) {
        // x[psi] += (dt/6)*(dx0 + dx1 + 4*0): the last stage leaves dx2[psi] = 0
        o.psi_rk = 1;
        o.psibase = plane(X, "psi");
        o.psi0 = plane(D[0], "psi");
        o.psi1 = nullptr;
        o.psiout = plane(X, "psi");
    } else if (inv2 && k == 2) {
        o.psi_rk = 1;
        o.psibase = plane(X, "psi");
        o.psi0 = plane(D[0], "psi");
        o.psi1 = plane(D[1], "psi");
        o.psiout = plane(X, "psi");
    }
    // Euler: u, v of the RK update are overwritten by the full solve
    if (kind != M_BOUSSINESQ && k == 2) o.rk = 0;
    return ortho(o, kind == M_QG, s);
}

// One RK3_SSP stage of the mixed form (see kernels_mixed.cu)
int Model::stage_mixed(int k, cudaStream_t s) {
    float *xs = k == 0 ? Xf : (k == 1 ? S1f : S2f);
    float *outf = k == 0 ? S1f : S2f;
    float *dk = Df[k];
    const char *tracers[2] = {kind == M_QG ? "pv" : "vorticity", "buoyancy"};
    const int ntr = kind == M_BOUSSINESQ ? 2 : 1;
    for (int t = 0; t < ntr; t++) {
        AdvMixed a;
        memset(&a, 0, sizeof(a));
        a.msk = msk;
        a.q = planef(xs, tracers[t]);
        a.u = planef(xs, "u");
        a.v = planef(xs, "v");
        a.advf = (const SplitT<float> *)advf;
        a.dtf = dtf;
        a.dq = planef(dk, tracers[t]);
        if (kind == M_BOUSSINESQ && t == 0) {
            a.buoy = planef(xs, "buoyancy");
            a.torque_coef = (float)(0.5 * desc.gravity / dx);
        }
        a.rk = k + 1;
        a.sbase = planef(Xf, tracers[t]);
        a.d0 = k >= 1 ? planef(Df[0], tracers[t]) : nullptr;
        a.d1 = k >= 2 ? planef(Df[1], tracers[t]) : nullptr;
        a.sout = k < 2 ? planef(outf, tracers[t]) : nullptr;
        a.xout = k == 2 ? plane(X, tracers[t]) : nullptr;
        a.kind = (desc.order % 2 == 0) ? 1 : 0;
        a.method = desc.flux_method;
        a.order = desc.order;
        a.mv = mv;
        a.nv = nv;
        if (k == 2) a.diff_coef = (float)diffusion_coef(t);
        TRY(stage_advection_mixed(a, s));
    }
    const bool inv = (kind == M_BOUSSINESQ) || k < 2 || (kind == M_EULER && desc.diffusion);
    if (!inv) return OK;
    double *psik = plane(D[k], "psi");
    if (kind == M_QG) TRY(cuda_status(cudaMemsetAsync(psik, 0, pl * 8, s), "qg warm start"));
    TRY(c2c_f32(planef(dk, tracers[0]), B, mv, nv, s));
    TRY(two_vcycle_mixed(gmg, psik, B, s));
    OrthoMixed o;
    memset(&o, 0, sizeof(o));
    o.msk = msk;
    o.mskp = mskp;
    o.psi = psik;
    o.du = planef(dk, "u");
    o.dv = planef(dk, "v");
    o.zdx = 1. / dx;
    o.zdy = 1. / dy;
    o.rk = k + 1;
    o.ubase = planef(Xf, "u");
    o.vbase = planef(Xf, "v");
    o.u0 = k >= 1 ? planef(Df[0], "u") : nullptr;
    o.v0 = k >= 1 ? planef(Df[0], "v") : nullptr;
    o.u1 = k >= 2 ? planef(Df[1], "u") : nullptr;
    o.v1 = k >= 2 ? planef(Df[1], "v") : nullptr;
    o.su = k < 2 ? planef(outf, "u") : nullptr;
    o.sv = k < 2 ? planef(outf, "v") : nullptr;
    o.xu = k == 2 ? plane(X, "u") : nullptr;
    o.xv = k == 2 ? plane(X, "v") : nullptr;
    if (!invert_at_forcing_stage() && k == 1) {
        o.psi_rk = 1;
        o.psibase = plane(X, "psi");
        o.psi0 = plane(D[0], "psi");
        o.psi1 = nullptr;
        o.psiout = plane(X, "psi");
    } else if (invert_at_forcing_stage() && k == 2) {
        o.psi_rk = 1;
        o.psibase = plane(X, "psi");
        o.psi0 = plane(D[0], "psi");
        o.psi1 = plane(D[1], "psi");
        o.psiout = plane(X, "psi");
    }
    o.dt = dt;
    o.dtf = dtf;
    o.mv = mv;
    o.nv = nv;
    return stage_ortho_mixed(o, s);
}

int Model::set_psi(cudaStream_t s) {
    if (kind == M_QG) {
        k_qg_post<<<blocks_for(pl), 256, 0, s>>>(X, pl, pvback, 0., 0);  // pvanom = pv - pvback
        TRY(launch_status("pvanom"));
        TRY(invert(X, "pvanom", true, s, true));
    } else {
        TRY(invert(X, "vorticity", true, s, true));
    }
    OrthoStage o = ortho_base(*this, X);
    return ortho(o, true, s);
}

int Model::diagnostics(cudaStream_t s) {
    DiagArgs a;
    a.kind = kind;
    a.msk = msk;
    a.s = X;
    a.pl = pl;
    a.mv = mv;
    a.nv = nv;
    a.dx = dx;
    a.dy = dy;
    a.gravity = desc.gravity;
    a.Rd = desc.Rd;
    a.area = area;
    a.part = part;
    a.out = diag;
    a.status = status;
    a.solve = gmg.solve_state;
    int rows = mv - 2 * NH;
    int nb = reduce_blocks(rows);
    int rpb = (rows + nb - 1) / nb;
    nb = (rows + rpb - 1) / rpb;
    a.nr = rpb;
    TRY(launch_body<BDiagP>(k_diag_partial, a, dim3(nb), dim3(RED_THREADS), 0, s, "diagnostics"));
    a.nr = nb;
    return launch_body<BDiagF>(k_diag_final, a, dim3(1), dim3(RED_THREADS), 0, s, "diagnostics");
}

// Fluid2d.loop body (core/fluid2d.py:237-268): set_dt, model.step, diagnostics
int Model::step(cudaStream_t s) {
    gmg.nprobe = 0;
    TRY(set_dt(dt, cst, advc, diag, desc.adaptable_dt, desc.dt, desc.cfl, dx < dy ? dx : dy,
               desc.dtmax, status, s));
    TRY(advance(s));
    return diagnostics(s);
}

// model.step after set_dt: the three stages and the post-step fields
int Model::advance(cudaStream_t s) {
    if (desc.precision != 0) {
        TRY(split_f32(advc, dt, advf, dtf, s));
        TRY(vec_to_f32(X, Xf, nvar * pl, s));
        for (int k = 0; k < 3; k++) TRY(stage_mixed(k, s));
    } else {
        for (int k = 0; k < 3; k++) TRY(stage(k, s));
    }
    if (noslip) TRY(add_noslip(s));
    if (kind == M_BOUSSINESQ) {
        TRY(launch_body<BBanom>(k_banom, BanomArgs{X, pl, bref}, dim3(blocks_for(pl)), dim3(256),
                                0, s, "banom"));
    } else {
        TRY(set_psi(s));
        if (kind == M_QG) {
            k_qg_post<<<blocks_for(pl), 256, 0, s>>>(X, pl, pvback, std::pow(desc.Rd, -2.0), 1);
            TRY(launch_status("qg post"));
        }
    }
    return OK;
}

// ---- no-slip walls
// core/operators.py:157-184: the boundary cells are the wall-mask cells with
// a solid neighbour (np.roll over the whole array), then the halo is filled
int Model::noslip_setup(const int8_t *mh, cudaStream_t s) {
    std::vector<int8_t> bc(pl, 0);
    for (int j = 0; j < mv; j++)
        for (int i = 0; i < nv; i++) {
            const int c = mh[off(j, i, nv)];
            const int z = mh[off(j, (i + 1) % nv, nv)] + mh[off((j + 1) % mv, i, nv)] +
                          mh[off(j, (i + nv - 1) % nv, nv)] + mh[off((j + mv - 1) % mv, i, nv)] -
                          4 * c;
            bc[off(j, i, nv)] = (z * c < 0) ? (int8_t)c : 0;
        }
    // fillhalo (periodic images of the interior, core/gmg/fortran_multigrid.f90:365-412)
    const int m2 = mv - 2 * NH, n2 = nv - 2 * NH;
    for (int j = 0; j < mv; j++)
        for (int i = 0; i < nv; i++) {
            int jj = j < NH ? j + m2 : (j >= mv - NH ? j - m2 : j);
            int ii = i < NH ? i + n2 : (i >= nv - NH ? i - n2 : i);
            if (jj != j || ii != i) bc[off(j, i, nv)] = bc[off(jj, ii, nv)];
        }
    double area = 0.;
    for (int j = NH; j < mv - NH; j++)
        for (int i = NH; i < nv - NH; i++) area += bc[off(j, i, nv)];
    if (!(area > 0)) {
        set_error("noslip: the wall mask has no boundary cell");
        return ERR_ARG;
    }
    Noslip *N = new (std::nothrow) Noslip();
    if (!N) return ERR_CUDA;
    size_t om = N->mem.add(pl), ob = N->mem.add(pl), os = N->mem.add(sizeof(double) * pl),
           ou = N->mem.add(sizeof(double) * 4);
    int st = N->mem.alloc();
    if (st) {
        delete N;
        return st;
    }
    N->msk = N->mem.at<int8_t>(om);
    N->mskbc = N->mem.at<int8_t>(ob);
    N->src = kind == M_EULER ? plane(X, "source") : N->mem.at<double>(os);
    N->sum = N->mem.at<double>(ou);
    N->bcarea = area;
    st = cuda_status(cudaMemcpyAsync(N->msk, mh, pl, cudaMemcpyHostToDevice, s), "noslip msk");
    if (!st)
        st = cuda_status(cudaMemcpyAsync(N->mskbc, bc.data(), pl, cudaMemcpyHostToDevice, s),
                         "noslip mskbc");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "noslip setup");
    if (st) {
        delete N;
        return st;
    }
    delete noslip;
    noslip = N;
    return OK;
}

// rhs_noslip then invert_vorticity(x, 'fast') on the state
// (core/euler.py:109-113, 171-179; core/boussinesq.py:93-94, 116-118;
// core/quasigeostrophic.py:112-114, 171-175); Euler keeps source/dt
int Model::add_noslip(cudaStream_t s) {
    Noslip &N = *noslip;
    const char *who = kind == M_QG ? "pvanom" : "vorticity";
    if (kind == M_QG) {
        const bool mixed = desc.precision != 0;
        TRY(pvanom_rk(plane(X, "pvanom"), mixed ? nullptr : plane(D[0], "pv"),
                      mixed ? nullptr : plane(D[1], "pv"), mixed ? planef(Df[0], "pv") : nullptr,
                      mixed ? planef(Df[1], "pv") : nullptr, dt, pl, s));
    }
    TRY(noslip_source(N.msk, plane(X, "psi"), N.src, dx, dy, mv, nv, s));
    // domain_integration(source) / bcarea, an unmasked sum over the interior
    TRY(launch_reduce(2, ones, N.src, nullptr, NH, mv, nv, N.sum, gmg.work, s));
    TRY(noslip_mean(N.src, N.sum, N.mskbc, N.bcarea, pl, s));
    TRY(launch_fillhalo(N.src, NH, mv, nv, s));
    TRY(plane_sub(plane(X, who), N.src, pl, s));
    TRY(invert(X, who, false, s, true));
    OrthoStage o = ortho_base(*this, X);
    TRY(ortho(o, true, s));
    if (kind == M_EULER) TRY(plane_div(N.src, dt, pl, s));
    return OK;
}

// ---- flux diagnostic (core/fluxes.py)
int Model::flux_setup(cudaStream_t s) {
    if (flux) return OK;
    if (kind == M_QG) {
        set_error("flux diagnostic: not available for the quasigeostrophic model "
                  "(core/fluxes.py:14-16)");
        return ERR_ARG;
    }
    Flux *F = new (std::nothrow) Flux();
    if (!F) return ERR_CUDA;
    const char *trn[4];
    F->ntr = 0;
    trn[F->ntr] = "vorticity";
    F->tr[F->ntr++] = (int)(plane(X, "vorticity") - X) / (int)pl;
    if (kind == M_BOUSSINESQ) {
        trn[F->ntr] = "buoyancy";
        F->tr[F->ntr++] = (int)((plane(X, "buoyancy") - X) / pl);
    }
    trn[F->ntr] = "uc";
    F->tr[F->ntr++] = nvar;
    trn[F->ntr] = "vc";
    F->tr[F->ntr++] = nvar + 1;
    F->ns = nvar + 2;
    F->nflx = 2 * F->ntr;
    F->next = F->ns + F->nflx;
    F->nfull = 2 * F->nflx;
    const char *rr[2] = {"rev", "irr"}, *dd[2] = {"x", "y"};
    for (int r = 0; r < 2; r++)
        for (int t = 0; t < F->ntr; t++)
            for (int d = 0; d < 2; d++)
                F->names.push_back(std::string(rr[r]) + "_" + dd[d] + "_" + trn[t]);
    const size_t ext = sizeof(double) * pl * F->next;
    size_t oX = F->mem.add(ext), oXw = F->mem.add(ext), oS = F->mem.add(ext);
    size_t oD[3] = {F->mem.add(ext), F->mem.add(ext), F->mem.add(ext)};
    size_t oXe = F->mem.add(sizeof(double) * pl * F->ns);
    size_t oF = F->mem.add(sizeof(double) * pl * F->nfull);
    size_t oc = F->mem.add(sizeof(double) * 8);
    int st = F->mem.alloc();
    if (st) {
        delete F;
        return st;
    }
    F->X = F->mem.at<double>(oX);
    F->Xw = F->mem.at<double>(oXw);
    F->S = F->mem.at<double>(oS);
    for (int k = 0; k < 3; k++) F->D[k] = F->mem.at<double>(oD[k]);
    F->Xe = F->mem.at<double>(oXe);
    F->FLX = F->mem.at<double>(oF);
    F->fcst = F->mem.at<double>(oc);
    flux = F;
    return cuda_status(cudaStreamSynchronize(s), "flux setup");
}

// Fluxes.advection (core/fluxes.py:172-213): flux-form advection of every
// quantity with its edge fluxes, the torque (Boussinesq), the fast inversion
int Model::flux_rhs(const double *xs, double *dxdt, cudaStream_t s) {
    Flux &F = *flux;
    const int iu = (int)((plane(X, "u") - X) / pl), iv = (int)((plane(X, "v") - X) / pl);
    const int ip = (int)((plane(X, "psi") - X) / pl), iw = F.tr[0];
    const int akind = (desc.order % 2 == 0) ? 2 : 0;
    for (int t = 0; t < F.ntr; t++) {
        const int ik = F.tr[t], ix = F.ns + 2 * t, iy = ix + 1;
        TRY(launch_advection(akind, msk, xs + ik * pl, dxdt + ik * pl, xs + iu * pl,
                             xs + iv * pl, dxdt + ix * pl, dxdt + iy * pl, F.fcst, NH,
                             desc.flux_method, desc.order, mv, nv, s));
        TRY(launch_fillhalo(dxdt + ik * pl, NH, mv, nv, s));
        TRY(launch_fillhalo(dxdt + ix * pl, NH, mv, nv, s));
        TRY(launch_fillhalo(dxdt + iy * pl, NH, mv, nv, s));
    }
    if (kind == M_BOUSSINESQ) {  // Operators.rhs_torque (core/operators.py:303-314)
        const int ib = F.tr[1];
        TRY(mul_mask(dxdt + iw * pl, msk, pl, s));
        TRY(launch_add_torque(msk, xs + ib * pl, dx, NH, desc.gravity, dxdt + iw * pl, mv, nv,
                              s));
        TRY(launch_fillhalo(dxdt + iw * pl, NH, mv, nv, s));
    }
    // Operators.invert_vorticity(dxdt, 'fast') (core/operators.py:421-498)
    double *psi = dxdt + ip * pl;
    TRY(launch_celltocorner(dxdt + iw * pl, B, mv, nv, s));
    TRY(two_vcycle(gmg, psi, B, s));
    TRY(mul_mask(psi, mskp, pl, s));
    return launch_orthogradient(msk, psi, dx, dy, mv, nv, dxdt + iu * pl, dxdt + iv * pl, s);
}

// Timescheme.forward = RK3_SSP (core/timescheme.py:167-180) of the extended
// state with dt * sgn
int Model::flux_forward(double sgn, cudaStream_t s) {
    Flux &F = *flux;
    const size_t n = pl * F.next;
    TRY(flux_rhs(F.X, F.D[0], s));
    TRY(flux_rk(0, n, F.X, F.D[0], F.D[1], F.D[2], F.S, dt, sgn, s));
    TRY(flux_rhs(F.S, F.D[1], s));
    TRY(flux_rk(1, n, F.X, F.D[0], F.D[1], F.D[2], F.S, dt, sgn, s));
    TRY(flux_rhs(F.S, F.D[2], s));
    return flux_rk(2, n, F.X, F.D[0], F.D[1], F.D[2], F.S, dt, sgn, s);
}

// Fluxes.diag_fluxes(state, t, dt) (core/fluxes.py:100-170) with the model's
// current dt and cst[3] (both on the device)
int Model::diag_fluxes(cudaStream_t s) {
    Flux &F = *flux;
    const int iu = (int)((plane(X, "u") - X) / pl), iv = (int)((plane(X, "v") - X) / pl);
    const int ip = (int)((plane(X, "psi") - X) / pl), iw = F.tr[0];
    TRY(cuda_status(cudaMemcpyAsync(F.Xe, X, sizeof(double) * pl * nvar,
                                    cudaMemcpyDeviceToDevice, s),
                    "flux state copy"));
    double *uc = F.Xe + (size_t)nvar * pl, *vc = uc + pl;
    TRY(flux_centre(X + iu * pl, X + iv * pl, uc, vc, mv, nv, s));
    TRY(launch_fillhalo(uc, NH, mv, nv, s));
    TRY(launch_fillhalo(vc, NH, mv, nv, s));
    TRY(flux_cst(F.fcst, cst, dx, dy, desc.aparab, s));
    TRY(flux_load(F.X, F.Xe, F.ns, F.next, pl, 0u, s));
    TRY(flux_forward(1., s));
    TRY(cuda_status(cudaMemcpyAsync(F.Xw, F.X, sizeof(double) * pl * F.next,
                                    cudaMemcpyDeviceToDevice, s),
                    "flux forward copy"));
    const unsigned neg = (1u << iu) | (1u << iv) | (1u << ip) | (1u << iw) | (1u << nvar) |
                         (1u << (nvar + 1));
    TRY(flux_load(F.X, F.Xe, F.ns, F.next, pl, neg, s));
    TRY(flux_forward(-1., s));
    return flux_final(F.nflx, F.ns, pl, F.Xw, F.X, F.FLX, dt, s);
}

// One iteration of core/fluid2d.py:235-311 on the device: set_dt with the
// exact-history-time adjustment, model.step, t += dt, diagnostics, Output.do
// into the rings, blow-up check.
int Model::loop_body(cudaStream_t s) {
    gmg.nprobe = 0;
    TRY(loop_pre(loop->clock, loop->k, dt, cst, advc, diag, s));
    TRY(advance(s));
    TRY(diagnostics(s));
    TRY(loop_post(loop->clock, loop->k, diag, loop->r, loop->h, loop->hflux, s));
    return loop_snapshot(loop->clock, loop->r, s);
}

// capture `body` into graph g after its current leaf nodes (none: at the root)
template <typename F>
static int capture_into(cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, cudaStream_t s,
                        F body) {
    TRY(cuda_status(cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(),
                                                  nullptr, deps.size(),
                                                  cudaStreamCaptureModeThreadLocal),
                    "capture begin"));
    int st = body();
    cudaGraph_t out = nullptr;
    int st2 = cuda_status(cudaStreamEndCapture(s, &out), "capture end");
    TRY(st);
    return st2;
}

// nodes of g without dependents
static int graph_leaves(cudaGraph_t g, std::vector<cudaGraphNode_t> &leaves) {
    size_t n = 0;
    TRY(cuda_status(cudaGraphGetNodes(g, nullptr, &n), "graph nodes"));
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) TRY(cuda_status(cudaGraphGetNodes(g, nodes.data(), &n), "graph nodes"));
    leaves.clear();
    for (size_t q = 0; q < n; q++) {
        size_t nd = 0;
        TRY(cuda_status(cudaGraphNodeGetDependentNodes(nodes[q], nullptr, nullptr, &nd),
                        "graph dependents"));
        if (nd == 0) leaves.push_back(nodes[q]);
    }
    return OK;
}

static int add_conditional(cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps,
                           cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                           cudaGraph_t *body) {
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    TRY(cuda_status(cudaGraphAddNode(&node, g, deps.empty() ? nullptr : deps.data(), nullptr,
                                     deps.size(), &p),
                    "conditional node"));
    *body = p.conditional.phGraph_out[0];
    return OK;
}

// Graph: gate kernel -> WHILE node { loop_body [-> IF node { flux diagnostic }] }.
// The gate and the last kernel of the body set the WHILE condition, which
// steps_left bounds in every launch; k_loop_post sets the IF condition when
// the step writes a history record.
int Model::loop_build(cudaStream_t s) {
    cudaGraph_t g = nullptr;
    TRY(cuda_status(cudaGraphCreate(&g, 0), "loop graph"));
    loop->graph = g;
    TRY(cuda_status(cudaGraphConditionalHandleCreate(&loop->h, g, 0, cudaGraphCondAssignDefault),
                    "loop condition"));
    std::vector<cudaGraphNode_t> deps;
    TRY(capture_into(g, deps, s, [&]() { return loop_gate(loop->clock, loop->k, loop->h, s); }));
    TRY(graph_leaves(g, deps));
    cudaGraph_t body = nullptr;
    TRY(add_conditional(g, deps, loop->h, cudaGraphCondTypeWhile, &body));
    if (loop->k.fluxes)
        TRY(cuda_status(cudaGraphConditionalHandleCreate(&loop->hflux, body, 0,
                                                         cudaGraphCondAssignDefault),
                        "flux condition"));
    deps.clear();
    TRY(capture_into(body, deps, s, [&]() { return loop_body(s); }));
    if (loop->k.fluxes) {
        TRY(graph_leaves(body, deps));
        cudaGraph_t fbody = nullptr;
        TRY(add_conditional(body, deps, loop->hflux, cudaGraphCondTypeIf, &fbody));
        deps.clear();
        TRY(capture_into(fbody, deps, s, [&]() {
            TRY(diag_fluxes(s));
            return loop_flux_snapshot(loop->clock, loop->r, s);
        }));
    }
    return cuda_status(cudaGraphInstantiate(&loop->exec, g, 0), "loop graph instantiate");
}

}  // namespace f2d

using namespace f2d;

extern "C" {

int f2d_model_create(const f2d_model_desc *d, const int8_t *msk_host, void **model) {
    if (!d || !msk_host || !model) {
        set_error("f2d_model_create: null argument");
        return ERR_ARG;
    }
    if (d->nx < 3 || d->ny < 3 || d->Lx <= 0 || d->Ly <= 0) {
        set_error("f2d_model_create: bad grid %dx%d", d->nx, d->ny);
        return ERR_SHAPE;
    }
    Model *M = new (std::nothrow) Model();
    if (!M) return ERR_CUDA;
    cudaStream_t s = nullptr;
    int st = M->create(d, msk_host, s);
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "model setup");
    if (st) {
        delete M;
        return st;
    }
    *model = M;
    return OK;
}

int f2d_model_destroy(void *model) {
    Model *M = (Model *)model;
    if (!M) return OK;
    if (M->gexec) cudaGraphExecDestroy(M->gexec);
    if (M->graph) cudaGraphDestroy(M->graph);
    M->drop_host_graph();
    delete M->loop;
    delete M->flux;
    delete M->noslip;
    delete M->isl;
    delete M;
    return OK;
}

int f2d_model_info(void *model, int *nvar, int *mv, int *nv, int *nlev, int *coarse_level,
                   double **state, double **diag) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    if (nvar) *nvar = M->nvar;
    if (mv) *mv = M->mv;
    if (nv) *nv = M->nv;
    if (nlev) *nlev = M->gmg.nlev;
    if (coarse_level) *coarse_level = M->gmg.cs;
    if (state) *state = M->X;
    if (diag) *diag = M->diag;
    return OK;
}

int f2d_model_bytes(void *model, size_t *bytes) {
    Model *M = (Model *)model;
    if (!M || !bytes) return ERR_ARG;
    *bytes = M->mem.total + M->gmg.mem.total;
    return OK;
}

const char *f2d_model_varname(void *model, int k) {
    Model *M = (Model *)model;
    if (!M || k < 0 || k >= M->nvar) return nullptr;
    return VARNAMES[M->kind][k];
}

const char *f2d_model_diagname(void *model, int k) {
    Model *M = (Model *)model;
    if (!M || k < 0 || k >= NDIAG[M->kind]) return nullptr;
    return DIAGNAMES[M->kind][k];
}

double *f2d_model_buffer(void *model, const char *which) {
    Model *M = (Model *)model;
    if (!M || !which) return nullptr;
    if (!strcmp(which, "state")) return M->X;
    if (!strcmp(which, "dx0")) return M->D[0];
    if (!strcmp(which, "dx1")) return M->D[1];
    if (!strcmp(which, "dx2")) return M->D[2];
    if (!strcmp(which, "cst")) return M->cst;
    if (!strcmp(which, "dt")) return M->dt;
    if (!strcmp(which, "diag")) return M->diag;
    if (!strcmp(which, "work")) return M->B;
    return nullptr;
}

int f2d_model_set_psi(void *model, void *stream) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    return M->set_psi((cudaStream_t)stream);
}

int f2d_model_diagnostics(void *model, void *stream) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    return M->diagnostics((cudaStream_t)stream);
}

int f2d_model_step(void *model, int nsteps, void *stream) {
    Model *M = (Model *)model;
    if (!M || nsteps < 0) return ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    for (int k = 0; k < nsteps; k++) TRY(M->step(s));
    return OK;
}

int f2d_model_set_dt(void *model, double dt) {
    Model *M = (Model *)model;
    if (!M || !(dt > 0)) return ERR_ARG;
    M->desc.dt = dt;
    if (M->gexec) {  // the captured step bakes dt in: capture again
        cudaGraphExecDestroy(M->gexec);
        cudaGraphDestroy(M->graph);
        M->gexec = nullptr;
        M->graph = nullptr;
    }
    M->drop_host_graph();
    if (M->loop) {
        M->loop->k.dt0 = dt;
        if (M->loop->exec) cudaGraphExecDestroy(M->loop->exec);
        if (M->loop->graph) cudaGraphDestroy(M->loop->graph);
        M->loop->exec = nullptr;
        M->loop->graph = nullptr;
    }
    return OK;
}

// Capture one step in a CUDA graph (on `stream`, which must not be the
// legacy default stream) and replay it nsteps times.
int f2d_model_step_graph(void *model, int nsteps, void *stream) {
    Model *M = (Model *)model;
    cudaStream_t s = (cudaStream_t)stream;
    if (!M || nsteps < 0 || !s) {
        set_error("f2d_model_step_graph: needs a model and a non-default stream");
        return ERR_ARG;
    }
    if (!M->gexec) {
        TRY(cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                        "begin capture"));
        int st = M->step(s);
        cudaGraph_t g = nullptr;
        int st2 = cuda_status(cudaStreamEndCapture(s, &g), "end capture");
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        TRY(st2);
        M->graph = g;
        TRY(cuda_status(cudaGraphInstantiate(&M->gexec, g, 0), "graph instantiate"));
    }
    for (int k = 0; k < nsteps; k++) TRY(cuda_status(cudaGraphLaunch(M->gexec, s), "graph launch"));
    return OK;
}

// nsteps steps of the model whose state lives in host memory `host`
// (page-locked, the state's layout: nvar planes of (ny+6) x (nx+6) float64):
// every step uploads it, steps and reads it back, the three captured as one
// graph (for this host buffer) and replayed, so that no host-side gap
// separates the copies from the step.
int f2d_model_step_host(void *model, int nsteps, double *host, void *stream) {
    Model *M = (Model *)model;
    cudaStream_t s = (cudaStream_t)stream;
    if (!M || nsteps < 0 || !s || !host) {
        set_error("f2d_model_step_host: needs a model, a host buffer and a non-default stream");
        return ERR_ARG;
    }
    if (M->hexec && M->hptr != host) M->drop_host_graph();
    if (!M->hexec) {
        const size_t bytes = (size_t)M->nvar * M->pl * sizeof(double);
        TRY(cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                        "begin capture"));
        int st = cuda_status(cudaMemcpyAsync(M->X, host, bytes, cudaMemcpyHostToDevice, s),
                             "state upload (the host buffer must be page-locked)");
        if (!st) st = M->step(s);
        if (!st)
            st = cuda_status(cudaMemcpyAsync(host, M->X, bytes, cudaMemcpyDeviceToHost, s),
                             "state read-back");
        cudaGraph_t g = nullptr;
        const int st2 = cuda_status(cudaStreamEndCapture(s, &g), "end capture");
        if (st || st2) {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            return st ? st : st2;
        }
        cudaGraphExec_t e = nullptr;
        const int st3 = cuda_status(cudaGraphInstantiate(&e, g, 0), "graph instantiate");
        if (st3) {
            cudaGraphDestroy(g);
            return st3;
        }
        M->hgraph = g;
        M->hexec = e;
        M->hptr = host;
    }
    for (int k = 0; k < nsteps; k++)
        TRY(cuda_status(cudaGraphLaunch(M->hexec, s), "graph launch"));
    return OK;
}

// Where the hierarchy switches to the single-CTA coarse solve: any level from
// the finest whose suffix fits the CTA's shared memory to nlev (no CTA).  The
// arithmetic is the same either way; only the launch structure changes.
// level < 0 only queries.
}  // extern "C"

// the captured step and loop graphs hold the old launch structure
static void drop_graphs(Model *M) {
    if (M->gexec) cudaGraphExecDestroy(M->gexec);
    if (M->graph) cudaGraphDestroy(M->graph);
    M->gexec = nullptr;
    M->graph = nullptr;
    M->drop_host_graph();
    if (M->loop) {
        if (M->loop->exec) cudaGraphExecDestroy(M->loop->exec);
        if (M->loop->graph) cudaGraphDestroy(M->loop->graph);
        M->loop->exec = nullptr;
        M->loop->graph = nullptr;
    }
}

// rebuild the coarse operators on a private stream and wait for them
static int rebuild_coarse_op(Gmg &g) {
    cudaStream_t s = nullptr;
    TRY(cuda_status(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "coarse op stream"));
    int st = g.build_coarse_op(s);
    const int st2 = cuda_status(cudaStreamSynchronize(s), "coarse op build");
    cudaStreamDestroy(s);
    return st ? st : st2;
}

extern "C" {

int f2d_model_coarse_level(void *model, int level, int *current, int *first, int *nlev) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    Gmg &g = M->gmg;
    if (level >= 0) {
        if (g.tri || level < g.cs_min || level > g.nlev) {
            set_error("f2d_model_coarse_level: level %d outside [%d, %d]", level, g.cs_min,
                      g.nlev);
            return ERR_ARG;
        }
        if (level != g.cs) {
            g.cs = level;
            drop_graphs(M);
            if (rebuild_coarse_op(g) != OK) {  // fall back to the coarse CTA
                g.free_coarse_op();
                (void)cudaGetLastError();
            }
        }
    }
    if (current) *current = g.cs;
    if (first) *first = g.cs_min;
    if (nlev) *nlev = g.nlev;
    return OK;
}

int f2d_model_reset_graphs(void *model) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    drop_graphs(M);
    return OK;
}

int f2d_model_coarse_op(void *model, int enable, int *n) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    Gmg &g = M->gmg;
    if (enable >= 0 && (enable != 0) != g.coarse_op) {
        g.coarse_op = enable != 0;
        drop_graphs(M);
        TRY(rebuild_coarse_op(g));
    }
    if (n) *n = g.op_n;
    return OK;
}

// the multigrid cycles' persisting L2 windows: 1 on (the default), 0 off;
// < 0 only queries; returns the previous setting.  Read when a step is
// launched or captured.
int f2d_set_l2_persist(int mode) {
    const int prev = l2_persist_mode();
    if (mode == 0 || mode == 1) l2_persist_mode() = mode;
    return prev;
}

// the float level from which the mixed form's small-level cycles run as one
// cluster launch (-1: none, or the switch off)
int f2d_model_cluster_level(void *model, int *level) {
    Model *M = (Model *)model;
    if (!M || !level) return ERR_ARG;
    const Gmg &g = M->gmg;
    *level = (g.cl_lev >= 0 && g.op_cs == g.cs && cluster_mode()) ? g.cl_lev : -1;
    return OK;
}

// ---- batched steps of many models (batch.cu)
static int batch_record_step(void *ctx, int i) { return ((Model **)ctx)[i]->step(nullptr); }

int f2d_batch_create(void **models, int n, int policy, void **batch) {
    if (!models || n < 1 || !batch || policy < 0 || policy > 1) {
        set_error("f2d_batch_create: bad argument");
        return ERR_ARG;
    }
    for (int i = 0; i < n; i++) {
        Model *M = (Model *)models[i];
        if (!M) return ERR_ARG;
        if (M->kind == M_QG || M->noslip || M->isl || M->gmg.tri || M->gmg.probe) {
            set_error("f2d_batch_create: model %d uses a feature without a batched form "
                      "(quasigeostrophic, no-slip walls, islands, line relaxation, probe)",
                      i);
            return ERR_ARG;
        }
    }
    return batch_create(n, batch_record_step, (void *)models, policy, batch);
}

int f2d_batch_step(void *batch, int nsteps, void *stream) {
    if (!batch || nsteps < 0) return ERR_ARG;
    return batch_step(batch, nsteps, (cudaStream_t)stream);
}

int f2d_batch_info(void *batch, int *launches, int *ops) {
    if (!batch) return ERR_ARG;
    return batch_info(batch, launches, ops);
}

int f2d_batch_destroy(void *batch) {
    if (batch) batch_destroy(batch);
    return OK;
}

// ---- islands (core/island.py, core/fluid2d.py:110-113)
int f2d_model_islands(void *model, const double *rhsp_host, const double *psi_host,
                      void *stream) {
    Model *M = (Model *)model;
    cudaStream_t s = (cudaStream_t)stream;
    if (!M || !rhsp_host || !psi_host) {
        set_error("f2d_model_islands: null argument");
        return ERR_ARG;
    }
    if (M->kind == M_QG && M->desc.precision != 0) {
        set_error("f2d_model_islands: the quasigeostrophic islands run in float64 only");
        return ERR_ARG;
    }
    Model::Islands *I = new (std::nothrow) Model::Islands();
    if (!I) return ERR_CUDA;
    size_t o1 = I->mem.add(sizeof(double) * M->pl), o2 = I->mem.add(sizeof(double) * M->pl);
    int st = I->mem.alloc();
    if (!st) {
        I->rhsp = I->mem.at<double>(o1);
        I->psi = I->mem.at<double>(o2);
        st = cuda_status(cudaMemcpyAsync(I->rhsp, rhsp_host, sizeof(double) * M->pl,
                                         cudaMemcpyHostToDevice, s),
                         "islands rhsp");
    }
    if (!st)
        st = cuda_status(cudaMemcpyAsync(I->psi, psi_host, sizeof(double) * M->pl,
                                         cudaMemcpyHostToDevice, s),
                         "islands psi");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "islands");
    if (st) {
        delete I;
        return st;
    }
    delete M->isl;
    M->isl = I;
    if (M->gexec) cudaGraphExecDestroy(M->gexec);
    if (M->graph) cudaGraphDestroy(M->graph);
    M->gexec = nullptr;
    M->graph = nullptr;
    if (M->loop) {
        if (M->loop->exec) cudaGraphExecDestroy(M->loop->exec);
        if (M->loop->graph) cudaGraphDestroy(M->loop->graph);
        M->loop->exec = nullptr;
        M->loop->graph = nullptr;
    }
    return OK;
}

// ---- no-slip walls (core/operators.py:245-290)
int f2d_model_noslip(void *model, const int8_t *msknoslip_host, void *stream) {
    Model *M = (Model *)model;
    if (!M || !msknoslip_host) {
        set_error("f2d_model_noslip: null argument");
        return ERR_ARG;
    }
    TRY(M->noslip_setup(msknoslip_host, (cudaStream_t)stream));
    // captured graphs hold the step without the wall source: capture again
    if (M->gexec) cudaGraphExecDestroy(M->gexec);
    if (M->graph) cudaGraphDestroy(M->graph);
    M->gexec = nullptr;
    M->graph = nullptr;
    if (M->loop) {
        if (M->loop->exec) cudaGraphExecDestroy(M->loop->exec);
        if (M->loop->graph) cudaGraphDestroy(M->loop->graph);
        M->loop->exec = nullptr;
        M->loop->graph = nullptr;
    }
    return OK;
}

// ---- flux diagnostic (core/fluxes.py:100-213)
int f2d_model_flux_setup(void *model, void *stream) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    return M->flux_setup((cudaStream_t)stream);
}

int f2d_model_diag_fluxes(void *model, void *stream) {
    Model *M = (Model *)model;
    if (!M || !M->flux) {
        set_error("f2d_model_diag_fluxes: call f2d_model_flux_setup first");
        return ERR_ARG;
    }
    return M->diag_fluxes((cudaStream_t)stream);
}

int f2d_model_flux_info(void *model, int *nfull, double **flx) {
    Model *M = (Model *)model;
    if (!M || !M->flux) return ERR_ARG;
    if (nfull) *nfull = M->flux->nfull;
    if (flx) *flx = M->flux->FLX;
    return OK;
}

const char *f2d_model_flux_name(void *model, int k) {
    Model *M = (Model *)model;
    if (!M || !M->flux || k < 0 || k >= M->flux->nfull) return nullptr;
    return M->flux->names[k].c_str();
}

// ---- device time loop (core/fluid2d.py:235-314, core/output.py:62-94)
int f2d_model_loop_setup(void *model, const f2d_loop_desc *ld, void *stream) {
    Model *M = (Model *)model;
    cudaStream_t s = (cudaStream_t)stream;
    if (!M || !ld) {
        set_error("f2d_model_loop_setup: null argument");
        return ERR_ARG;
    }
    if (ld->nsave < 0 || ld->nsave > LOOP_MAX_SAVE || ld->his_cap < 1 || ld->diag_cap < 1 ||
        !(ld->freq_his > 0) || !(ld->freq_diag > 0) || ld->rescaledtime < 0 ||
        ld->rescaledtime > 1) {
        set_error("f2d_model_loop_setup: bad loop description");
        return ERR_ARG;
    }
    for (int q = 0; q < ld->nsave; q++)
        if (ld->save[q] < 0 || ld->save[q] >= M->nvar) {
            set_error("f2d_model_loop_setup: saved plane %d out of range", ld->save[q]);
            return ERR_ARG;
        }
    // rescaledtime reads 'enstrophy' (core/fluid2d.py:258), which QG lacks
    if (ld->rescaledtime && M->kind == M_QG) {
        set_error("f2d_model_loop_setup: rescaledtime 'enstrophy' needs an enstrophy diagnostic");
        return ERR_ARG;
    }
    if (ld->diag_fluxes) TRY(M->flux_setup(s));
    delete M->loop;
    M->loop = new (std::nothrow) Model::Loop();
    if (!M->loop) return ERR_CUDA;
    Model::Loop &L = *M->loop;
    const int nfull = ld->diag_fluxes ? M->flux->nfull : 0;
    const int nd = NDIAG[M->kind];
    const size_t per = (size_t)M->desc.ny * M->desc.nx * (ld->nsave > 0 ? ld->nsave : 1);
    size_t o_clock = L.mem.add(sizeof(LoopClock));
    size_t o_his = L.mem.add(sizeof(float) * per * ld->his_cap);
    size_t o_ht = L.mem.add(sizeof(double) * ld->his_cap);
    size_t o_hk = L.mem.add(sizeof(int) * ld->his_cap);
    size_t o_diag = L.mem.add(sizeof(double) * (size_t)(nd + 4) * ld->diag_cap);
    size_t o_flx = L.mem.add(sizeof(float) * (size_t)M->desc.ny * M->desc.nx * nfull *
                             ld->his_cap);
    TRY(L.mem.alloc());
    L.clock = L.mem.at<LoopClock>(o_clock);
    L.k.adaptable = M->desc.adaptable_dt;
    L.k.exacthistime = ld->exacthistime;
    L.k.rescale = ld->rescaledtime;
    L.k.ike = 1;
    L.k.iens = M->kind == M_EULER ? 3 : (M->kind == M_BOUSSINESQ ? 5 : 3);
    L.k.ndiag = nd;
    L.k.his_cap = ld->his_cap;
    L.k.diag_cap = ld->diag_cap;
    L.k.dt0 = M->desc.dt;
    L.k.cfl = M->desc.cfl;
    L.k.hmin = M->dx < M->dy ? M->dx : M->dy;
    L.k.dtmax = M->desc.dtmax;
    L.r.his = L.mem.at<float>(o_his);
    L.r.his_t = L.mem.at<double>(o_ht);
    L.r.his_kt = L.mem.at<int>(o_hk);
    L.r.diag = L.mem.at<double>(o_diag);
    L.r.X = M->X;
    L.r.pl = M->pl;
    L.r.mv = M->mv;
    L.r.nv = M->nv;
    L.r.nsave = ld->nsave;
    for (int q = 0; q < ld->nsave; q++) L.r.planes[q] = ld->save[q];
    L.k.fluxes = ld->diag_fluxes ? 1 : 0;
    L.r.nfull = nfull;
    L.r.flx = nfull ? L.mem.at<float>(o_flx) : nullptr;
    L.r.FLX = nfull ? M->flux->FLX : nullptr;
    LoopClock c;
    memset(&c, 0, sizeof(c));
    c.t = ld->t;
    c.dt = M->desc.dt;
    c.tend = ld->tend;
    c.tnexthis = ld->tnexthis;
    c.tnextdiag = ld->tnextdiag;
    c.freq_his = ld->freq_his;
    c.freq_diag = ld->freq_diag;
    c.kt = ld->kt;
    c.his_slot = -1;
    c.status = LOOP_RUNNING;
    TRY(cuda_status(cudaMemcpyAsync(L.clock, &c, sizeof(c), cudaMemcpyHostToDevice, s),
                    "loop clock"));
    return cuda_status(cudaStreamSynchronize(s), "loop setup");
}

// the loop's start (core/fluid2d.py:199-214): diagnostics and Output.do at t
int f2d_model_loop_start(void *model, void *stream) {
    Model *M = (Model *)model;
    if (!M || !M->loop) {
        set_error("f2d_model_loop_start: no loop set up");
        return ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    TRY(M->diagnostics(s));
    if (M->loop->k.fluxes) {
        // set_dt then the flux diagnostic (core/fluid2d.py:203-210)
        TRY(set_dt(M->dt, M->cst, M->advc, M->diag, M->desc.adaptable_dt, M->desc.dt,
                   M->desc.cfl, M->dx < M->dy ? M->dx : M->dy, M->desc.dtmax, M->status, s));
        TRY(M->diag_fluxes(s));
    }
    TRY(loop_record(M->loop->clock, M->loop->k, M->diag, M->loop->r, s));
    TRY(loop_snapshot(M->loop->clock, M->loop->r, s));
    return loop_flux_snapshot(M->loop->clock, M->loop->r, s);
}

// Run steps until t >= tend, a blow-up, a full ring or max_steps steps,
// whichever comes first, as one graph launch (no host synchronisation).  The
// graph is captured once, on a private stream, and launched on `stream`.
int f2d_model_loop_run(void *model, int max_steps, void *stream) {
    Model *M = (Model *)model;
    cudaStream_t s = (cudaStream_t)stream;
    if (!M || !M->loop || max_steps < 0) {
        set_error("f2d_model_loop_run: needs a loop set up and max_steps >= 0");
        return ERR_ARG;
    }
    if (M->gmg.probe) {
        set_error("f2d_model_loop_run: disable the smoother probe first");
        return ERR_ARG;
    }
    Model::Loop &L = *M->loop;
    if (!L.exec) {
        if (!L.capture)
            TRY(cuda_status(cudaStreamCreateWithFlags(&L.capture, cudaStreamNonBlocking),
                            "loop capture stream"));
        int st = M->loop_build(L.capture);
        if (st) {
            if (L.exec) cudaGraphExecDestroy(L.exec);
            if (L.graph) cudaGraphDestroy(L.graph);
            L.exec = nullptr;
            L.graph = nullptr;
            return st;
        }
    }
    TRY(cuda_status(cudaMemcpyAsync(&L.clock->steps_left, &max_steps, sizeof(int),
                                    cudaMemcpyHostToDevice, s),
                    "loop steps"));
    return cuda_status(cudaGraphLaunch(L.exec, s), "loop graph launch");
}

int f2d_model_loop_state(void *model, f2d_loop_state *out, void *stream) {
    Model *M = (Model *)model;
    cudaStream_t s = (cudaStream_t)stream;
    if (!M || !M->loop || !out) return ERR_ARG;
    LoopClock c;
    TRY(cuda_status(cudaMemcpyAsync(&c, M->loop->clock, sizeof(c), cudaMemcpyDeviceToHost, s),
                    "loop state"));
    TRY(cuda_status(cudaStreamSynchronize(s), "loop state sync"));
    out->t = c.t;
    out->dt = c.dt;
    out->tnexthis = c.tnexthis;
    out->tnextdiag = c.tnextdiag;
    out->kt = c.kt;
    out->status = c.status;
    out->nhis = c.nhis;
    out->ndiag = c.ndiag;
    return OK;
}

// Copy the records waiting in the rings to host memory and empty the rings.
// his: nhis x nsave x ny x nx float32; his_t, his_kt: nhis; diag_rows:
// ndiag x (ndiag_values + 4) float64.  Null outputs are skipped.
int f2d_model_loop_drain(void *model, float *his, float *flx, double *his_t, int *his_kt,
                         double *diag_rows, int *nhis, int *ndiag, void *stream) {
    Model *M = (Model *)model;
    cudaStream_t s = (cudaStream_t)stream;
    if (!M || !M->loop) return ERR_ARG;
    Model::Loop &L = *M->loop;
    LoopClock c;
    TRY(cuda_status(cudaMemcpyAsync(&c, L.clock, sizeof(c), cudaMemcpyDeviceToHost, s),
                    "loop drain"));
    TRY(cuda_status(cudaStreamSynchronize(s), "loop drain sync"));
    const size_t per = (size_t)M->desc.ny * M->desc.nx * L.r.nsave;
    if (his && c.nhis && per)
        TRY(cuda_status(cudaMemcpyAsync(his, L.r.his, sizeof(float) * per * c.nhis,
                                        cudaMemcpyDeviceToHost, s),
                        "loop drain his"));
    const size_t fper = (size_t)M->desc.ny * M->desc.nx * L.r.nfull;
    if (flx && c.nhis && fper)
        TRY(cuda_status(cudaMemcpyAsync(flx, L.r.flx, sizeof(float) * fper * c.nhis,
                                        cudaMemcpyDeviceToHost, s),
                        "loop drain flx"));
    if (his_t && c.nhis)
        TRY(cuda_status(cudaMemcpyAsync(his_t, L.r.his_t, sizeof(double) * c.nhis,
                                        cudaMemcpyDeviceToHost, s),
                        "loop drain his_t"));
    if (his_kt && c.nhis)
        TRY(cuda_status(cudaMemcpyAsync(his_kt, L.r.his_kt, sizeof(int) * c.nhis,
                                        cudaMemcpyDeviceToHost, s),
                        "loop drain his_kt"));
    if (diag_rows && c.ndiag)
        TRY(cuda_status(cudaMemcpyAsync(diag_rows, L.r.diag,
                                        sizeof(double) * (size_t)(L.k.ndiag + 4) * c.ndiag,
                                        cudaMemcpyDeviceToHost, s),
                        "loop drain diag"));
    const int zero[2] = {0, 0};
    TRY(cuda_status(cudaMemcpyAsync(&L.clock->nhis, zero, sizeof(zero), cudaMemcpyHostToDevice, s),
                    "loop drain reset"));
    TRY(cuda_status(cudaStreamSynchronize(s), "loop drain sync"));
    if (nhis) *nhis = c.nhis;
    if (ndiag) *ndiag = c.ndiag;
    return OK;
}

// Finest-level smoother probe: enable (resets the count; a captured graph is
// dropped so that the next capture records the probe events), or read the
// average duration (ms) of the probed smooth calls of the last step.
int f2d_model_probe(void *model, int enable, int *count, double *avg_ms) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    if (enable >= 0) {
        M->gmg.probe = enable != 0;
        M->gmg.nprobe = 0;
        M->probe_per_step = -1;
        if (M->gexec) {
            cudaGraphExecDestroy(M->gexec);
            cudaGraphDestroy(M->graph);
            M->gexec = nullptr;
            M->graph = nullptr;
        }
        return OK;
    }
    int n = M->gmg.nprobe;
    double tot = 0.;
    for (int k = 0; k < n; k++) {
        float ms = 0.f;
        TRY(cuda_status(cudaEventElapsedTime(&ms, M->gmg.ev[k][0], M->gmg.ev[k][1]), "probe time"));
        tot += ms;
    }
    if (count) *count = n;
    if (avg_ms) *avg_ms = n ? tot / n : 0.;
    return OK;
}

// kernel nodes of the captured step graph (0 before the first capture)
int f2d_model_graph_kernels(void *model, int *nkernels) {
    Model *M = (Model *)model;
    if (!M || !nkernels) return ERR_ARG;
    *nkernels = 0;
    if (!M->graph) return OK;
    size_t n = 0;
    TRY(cuda_status(cudaGraphGetNodes(M->graph, nullptr, &n), "graph nodes"));
    std::vector<cudaGraphNode_t> nodes(n);
    TRY(cuda_status(cudaGraphGetNodes(M->graph, nodes.data(), &n), "graph nodes"));
    int k = 0;
    for (size_t q = 0; q < n; q++) {
        cudaGraphNodeType t;
        TRY(cuda_status(cudaGraphNodeGetType(nodes[q], &t), "node type"));
        if (t == cudaGraphNodeTypeKernel) k++;
    }
    *nkernels = k;
    return OK;
}

int f2d_model_status(void *model, int clear, int *status, void *stream) {
    Model *M = (Model *)model;
    if (!M || !status) {
        set_error("f2d_model_status: null argument");
        return ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int v = 0;
    TRY(cuda_status(cudaMemcpyAsync(&v, M->status, sizeof(int), cudaMemcpyDeviceToHost, s),
                    "status read"));
    if (clear) TRY(cuda_status(cudaMemsetAsync(M->status, 0, sizeof(int), s), "status clear"));
    TRY(cuda_status(cudaStreamSynchronize(s), "status sync"));
    *status = v;
    return OK;
}

// the status words of many models with one synchronisation: every word is
// copied into a pinned host buffer owned by the library, then the stream is
// synchronised once
int f2d_models_status(void **models, int n, int clear, int *status, void *stream) {
    if (n < 0 || (n > 0 && (!models || !status))) {
        set_error("f2d_models_status: bad argument");
        return ERR_ARG;
    }
    static std::mutex mu;
    static int *pinned = nullptr;
    static int cap = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (n > cap) {
        if (pinned) cudaFreeHost(pinned);
        pinned = nullptr;
        cap = 0;
        const int want = n < 1024 ? 1024 : n;
        TRY(cuda_status(cudaHostAlloc((void **)&pinned, want * sizeof(int), cudaHostAllocDefault),
                        "status buffer"));
        cap = want;
    }
    cudaStream_t s = (cudaStream_t)stream;
    for (int k = 0; k < n; k++) {
        Model *M = (Model *)models[k];
        if (!M) {
            set_error("f2d_models_status: null model %d", k);
            return ERR_ARG;
        }
        TRY(cuda_status(cudaMemcpyAsync(pinned + k, M->status, sizeof(int),
                                        cudaMemcpyDeviceToHost, s), "status read"));
        if (clear)
            TRY(cuda_status(cudaMemsetAsync(M->status, 0, sizeof(int), s), "status clear"));
    }
    TRY(cuda_status(cudaStreamSynchronize(s), "status sync"));
    for (int k = 0; k < n; k++) status[k] = pinned[k];
    return OK;
}

int f2d_model_solve_stats(void *model, int *nite, double *res, int *status) {
    Model *M = (Model *)model;
    if (!M) return ERR_ARG;
    SolveState st;
    TRY(cuda_status(cudaMemcpy(&st, M->gmg.solve_state, sizeof(st), cudaMemcpyDeviceToHost),
                    "solve stats"));
    if (nite) *nite = st.nite;
    if (res) *res = st.res;
    if (status) *status = st.status;
    return OK;
}

// ---- multigrid on caller arrays (core/gmg/hierarchy.py:154-218)
int f2d_gmg_create(const int8_t *mskp_host, int nx, int ny, double dx, double dy,
                   double hydroepsilon, int qg, double Rd, void **gmg) {
    if (!mskp_host || !gmg || nx < 3 || ny < 3) {
        set_error("f2d_gmg_create: bad argument");
        return ERR_ARG;
    }
    Gmg *G = new (std::nothrow) Gmg();
    if (!G) return ERR_CUDA;
    int st = G->setup(mskp_host, nx, ny, dx, dy, qg ? 1. : hydroepsilon, 8. / 9., qg != 0, Rd,
                      false, nullptr);
    if (!st) st = cuda_status(cudaDeviceSynchronize(), "gmg setup");
    if (st) {
        delete G;
        return st;
    }
    *gmg = G;
    return OK;
}

int f2d_gmg_destroy(void *gmg) {
    delete (Gmg *)gmg;
    return OK;
}

int f2d_gmg_levels(void *gmg, int *nlev, int *mv, int *nv, int *coarse_level) {
    Gmg *G = (Gmg *)gmg;
    if (!G) return ERR_ARG;
    if (nlev) *nlev = G->nlev;
    for (int l = 0; l < G->nlev; l++) {
        if (mv) mv[l] = G->mv[l];
        if (nv) nv[l] = G->nv[l];
    }
    if (coarse_level) *coarse_level = G->cs;
    return OK;
}

int f2d_gmg_twovcycle(void *gmg, double *x, const double *b, void *stream) {
    Gmg *G = (Gmg *)gmg;
    if (!G || !x || !b) return ERR_ARG;
    return two_vcycle(*G, x, b, (cudaStream_t)stream);
}

int f2d_gmg_solve(void *gmg, double *x, const double *b, int maxite, double tol, void *stream) {
    Gmg *G = (Gmg *)gmg;
    if (!G || !x || !b || maxite < 0) return ERR_ARG;
    return solve(*G, x, b, maxite, tol, (cudaStream_t)stream);
}

int f2d_gmg_solve_stats(void *gmg, int *nite, double *res, int *status) {
    Gmg *G = (Gmg *)gmg;
    if (!G) return ERR_ARG;
    SolveState st;
    TRY(cuda_status(cudaMemcpy(&st, G->solve_state, sizeof(st), cudaMemcpyDeviceToHost),
                    "solve stats"));
    if (nite) *nite = st.nite;
    if (res) *res = st.res;
    if (status) *status = st.status;
    return OK;
}

// level data: which = "msk" (int8), "A" (6 planes), "x", "b", "r"
void *f2d_gmg_level_ptr(void *gmg, int lev, const char *which) {
    Gmg *G = (Gmg *)gmg;
    if (!G || lev < 0 || lev >= G->nlev || !which) return nullptr;
    LevelView<double> &L = G->d[lev];
    if (!strcmp(which, "msk")) return (void *)L.msk;
    if (!strcmp(which, "A")) return (void *)L.A;
    if (!strcmp(which, "x")) return L.x;
    if (!strcmp(which, "b")) return L.b;
    if (!strcmp(which, "r")) return L.r;
    return nullptr;
}

int f2d_gmg_vcycle(void *gmg, int lev1, void *stream) {
    Gmg *G = (Gmg *)gmg;
    if (!G || lev1 < 0 || lev1 >= G->nlev) return ERR_ARG;
    return G->vcycle(G->d, lev1, false, nullptr, (cudaStream_t)stream);
}

int f2d_gmg_fcycle(void *gmg, int lev1, void *stream) {
    Gmg *G = (Gmg *)gmg;
    if (!G || lev1 < 0 || lev1 >= G->nlev) return ERR_ARG;
    return G->fcycle(G->d, lev1, nullptr, (cudaStream_t)stream);
}

}  // extern "C"
