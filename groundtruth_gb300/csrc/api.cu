// Host driver and C ABI of the solver (include/gt_gb300.h).
//
// A solve (GroundTruth: PlaneStack._solve + _gmres, peec.py:2560-2607, 3093-3224) runs as FP64 iterative
// refinement around FP32 restarted GMRES: per column
//     r = b - K x                     FP64 system product (FP64 FFTs), the true residual
//     stop when ||r|| <= tol ||b||    the reference's stopping rule (peec.py:3119, 3132)
//     GMRES on K M^-1 u = r / ||r||   FP32 products and preconditioner, FP64 Hessenberg / Givens, up to
//                                     `restart` iterations or the cycle's target
//     x += ||r|| M^-1 (V y)           accumulated in FP64
// precision = 1 runs the same loop with an FP64 inner GMRES (the plain all-FP64 comparator).  Columns are
// batched: every kernel launch covers all columns still iterating, the factor of a frequency is read once
// per group of columns that share it.
#include "../../include/gt_gb300.h"
#include "solver.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace gt {

static thread_local std::string t_last_error;
std::atomic<long long> g_launches{0};
void set_error(const std::string& s) { t_last_error = s; }

void raise_smem(const void* fn, size_t bytes) {
    if (bytes <= 48 * 1024) return;
    static std::mutex lock;
    static std::map<std::pair<int, const void*>, size_t> cap;
    int dev = 0;
    GT_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(lock);
    size_t& c = cap[{dev, fn}];
    if (bytes <= c) return;
    GT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    c = bytes;
}

struct Invalid : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// a bounded device wait that gave up (GT_TIMEOUT)
struct Timeout : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// after a call's kernels have finished: did a TMA wait of the L_p pass give up?
static void check_device_waits() {
    if (lp_take_wait_timeouts())
        throw Timeout("a TMA load of the L_p product's FFT grid did not arrive within its wait limit");
}

// Device allocations owned by an object, freed together.
struct Pool {
    std::vector<void*> ptrs;
    bool dry = false;      // count the bytes only (memory planning), allocate nothing
    size_t bytes = 0;
    template <typename T> T* alloc(size_t n) {
        void* p = nullptr;
        if (n == 0) n = 1;
        bytes += n * sizeof(T);
        if (dry) return nullptr;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e != cudaSuccess) throw CudaError{e, "cudaMalloc of " + std::to_string(n * sizeof(T)) + " bytes"};
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    // on a stream: ordered before that stream's kernels (a pageable cudaMemcpy may still be landing when it
    // returns, ordered only on the legacy default stream)
    template <typename T> T* upload(const T* h, size_t n, cudaStream_t st) {
        T* d = alloc<T>(n);
        if (n && h) GT_CUDA(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
        return d;
    }
    template <typename T> T* upload(const T* h, size_t n) {
        T* d = alloc<T>(n);
        if (n && h) GT_CUDA(cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice));
        return d;
    }
    void release() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
    }
    ~Pool() { release(); }
};

// Per-kernel-family timing with CUDA events on the launch stream (gt_profile).
struct Profiler {
    // a geometry's solves and its operator sets' factorisations may run at once on two host threads: the
    // records are kept under a lock, and each flush settles only the regions of its own stream
    bool on = false;
    bool levels = false;   // also time each elimination level of the triangular solves
    struct Rec {
        int fam;
        cudaEvent_t a, b;
        double bytes;
        cudaStream_t st;
    };
    std::mutex lock;
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> free_events;
    std::vector<std::string> names;
    struct Acc {
        double ms = 0, bytes = 0;
        int launches = 0;
    };
    std::map<int, Acc> acc;
    int family(const char* n) {
        std::lock_guard<std::mutex> lk(lock);
        for (size_t i = 0; i < names.size(); ++i)
            if (names[i] == n) return (int)i;
        names.push_back(n);
        return (int)names.size() - 1;
    }
    cudaEvent_t ev() {
        {
            std::lock_guard<std::mutex> lk(lock);
            if (!free_events.empty()) {
                cudaEvent_t e = free_events.back();
                free_events.pop_back();
                return e;
            }
        }
        cudaEvent_t e;
        GT_CUDA(cudaEventCreate(&e));
        return e;
    }
    void push(const Rec& r) {
        std::lock_guard<std::mutex> lk(lock);
        pending.push_back(r);
    }
    void flush(cudaStream_t st) {
        std::lock_guard<std::mutex> lk(lock);
        std::vector<Rec> keep;
        for (auto& r : pending) {
            if (r.st != st) {
                keep.push_back(r);
                continue;
            }
            float ms = 0;
            GT_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
            auto& a = acc[r.fam];
            a.ms += ms;
            a.launches += 1;
            a.bytes += r.bytes;
            free_events.push_back(r.a);
            free_events.push_back(r.b);
        }
        pending.swap(keep);
    }
    ~Profiler() {
        for (auto& r : pending) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (auto e : free_events) cudaEventDestroy(e);
    }
};

// A CUDA-event region of a kernel family on a stream (a no-op while the profiler is off).
struct Scope {
    Profiler* p;
    int fam;
    cudaEvent_t a{};
    cudaStream_t st;
    double bytes;
    Scope(Profiler* prof, const char* name, cudaStream_t s, double algo_bytes = 0)
        : p(prof && prof->on ? prof : nullptr), fam(0), st(s), bytes(algo_bytes) {
        if (!p) return;
        fam = p->family(name);
        a = p->ev();
        GT_CUDA(cudaEventRecord(a, st));
    }
    ~Scope() {
        if (!p) return;
        try {
            cudaEvent_t b = p->ev();
            if (cudaEventRecord(b, st) == cudaSuccess) p->push({fam, a, b, bytes, st});
        } catch (...) {
        }
    }
};

struct Orient {
    int n0, n1, P0, P1, di, dj;
    int ld0;                                // the FFT grid's row stride: n0 rounded up to a multiple of 16
    int64_t off;
    int rows[2] = {0, 0}, bt[2] = {0, 0};   // tuned launch shapes per precision (0: not tuned)
    float* spec32;
    double* spec64;
    c32 *tw0_32, *tw1_32;
    c64 *tw0_64, *tw1_64;
};

struct Workspace {
    Pool pool;
    int ncol = 0, m = 0, prec = -1;
    // FP64 per column
    c64 *x64 = nullptr, *r64 = nullptr, *b64 = nullptr, *T64 = nullptr;
    double *rho = nullptr, *bnorm = nullptr;
    c64* npart = nullptr;
    c64* npart_k = nullptr;
    c64* nred = nullptr;
    // inner (precision R) per slot
    void *V = nullptr, *w = nullptr, *z = nullptr, *T = nullptr, *zfac = nullptr, *yfac = nullptr, *uvec = nullptr,
         *sd = nullptr, *vcur = nullptr;
    c64* partial = nullptr;
    // precision 3: the FP32 inner solve's preconditioner applied in FP64 (input, output and the sweeps' vectors)
    c64 *pr64 = nullptr, *pz64 = nullptr, *zfac64 = nullptr, *yfac64 = nullptr, *uvec64 = nullptr, *sd64 = nullptr;
    GmresState st{};
    int *slot_col = nullptr, *slot_op = nullptr, *g_ptr = nullptr, *g_slot = nullptr, *g_op = nullptr, *col_op = nullptr;
    int* slot_pc = nullptr;      // each slot's factorisation (the preconditioner's tables, panels and pivots)
    int* act = nullptr;
    int* act_host = nullptr;
    // outer GCR: directions P (corrections) and Q = K P, per column, k-major; step sizes; active columns
    int kmax = 0;
    c64 *gP = nullptr, *gQ = nullptr, *gbeta = nullptr, *galpha = nullptr, *gnu2 = nullptr;
    int* colact = nullptr;
    int* flag_dev = nullptr;
    int* flag_host = nullptr;
    int* its_col = nullptr;
    ~Workspace() {
        if (flag_host) cudaFreeHost(flag_host);
        if (act_host) cudaFreeHost(act_host);
    }
};

}  // namespace gt

using namespace gt;

struct gt_geometry {
    Geo geo{};
    Orient o[2]{};
    Fronts F{};
    Pool pool;
    std::vector<int64_t> level_ptr;
    std::vector<int> level_maxnf, level_maxnown;
    std::vector<double> level_panel;   // panel entries (sum of nf x nown) of each level
    int max_nf = 0;
    int64_t* d_order = nullptr;
    // the factorisation's order: each level's small fronts, then its large ones (nf >= tiled_nf, the blocked
    // multi-CTA elimination), with the large ones' counts and extents per level
    int64_t* d_forder = nullptr;
    std::vector<int> level_nbig, level_bigmaxnf, level_bigmaxnown, level_smallmaxnf;
    int tiled_nf = 256;
    // every large front (all levels), for the blocked selective inversion
    int64_t* d_bigfronts = nullptr;
    int nbig = 0, bigmax_nf = 1, bigmax_nown = 1;
    int64_t n_compact = 0, n_strips = 0;
    int64_t* d_c2d = nullptr;
    int64_t* d_sterm_ptr = nullptr;
    int* d_sterm_tab = nullptr;
    double* d_sterm_coef = nullptr;
    int64_t maxT = 0;  // largest S * P1 * ld0 of the two orientations
    int device = 0;    // the CUDA device the geometry's buffers live on (current at gt_geometry_create)
    // the last n_lowrank branches are left out of the S-term map: a derived stack whose operators come from
    // gt_operators_derive (its base's factorisations plus a low-rank update)
    int n_lowrank = 0;
    int ntw = 0;                 // split layers (face couplings per operator)
    Narrow narrow{};
    std::vector<int> h_branch_nodes;
    uint64_t fsig = 0;  // signature of the factor structure (ordering, fronts, panel layout)
    std::unique_ptr<Workspace> ws;
    Profiler prof;
    std::mutex lock;
    // the triangular sweeps of independent column groups run on these streams side by side, so that one
    // group's elimination level overlaps another's
    static constexpr int NSUB = 4;
    cudaStream_t sub[NSUB]{};
    cudaEvent_t fork{}, join[NSUB]{};
    void make_streams() {
        if (fork) return;
        GT_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        for (int k = 0; k < NSUB; ++k) {
            GT_CUDA(cudaStreamCreateWithFlags(&sub[k], cudaStreamNonBlocking));
            GT_CUDA(cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming));
        }
    }
    ~gt_geometry() {
        for (int k = 0; k < NSUB; ++k) {
            if (sub[k]) cudaStreamDestroy(sub[k]);
            if (join[k]) cudaEventDestroy(join[k]);
        }
        if (fork) cudaEventDestroy(fork);
    }
};

struct gt_operators {
    gt_geometry* g = nullptr;
    int nops = 0;
    // the factorisations: nfact of them; operator q is preconditioned by factorisation fslot[q] (its own, or
    // one borrowed from another operator); the tables, panels and pivots below are per factorisation
    int nfact = 0;
    std::vector<int> fslot;
    Pool pool;
    double* omega = nullptr;
    c64 *zs = nullptr, *zcap = nullptr, *zbr = nullptr, *tab = nullptr;
    c64* zmut = nullptr;         // [op][ntw] the split layers' face couplings
    c32* tab32 = nullptr;        // the admittance table rounded to FP32 (the FP32 preconditioner's stencils)
    // per front P = [Linv_own; -L_bnd Linv_own] (nf x nown) and the pivot reciprocals dinv ([op][nfac])
    c64* panel64 = nullptr;      // column-major per front (forward solves)
    c32* panel32 = nullptr;
    c64* panel64_rm = nullptr;   // row-major copies (backward solves)
    c32* panel32_rm = nullptr;
    c64* dinv64 = nullptr;
    c32* dinv32 = nullptr;
    std::vector<int> own;        // the operator whose frequency each factorisation was made at
    // per factorisation: its branch or capacitance admittances exceed its strips' by more than STIFF_RATIO, so
    // that FP32 node potentials cannot resolve the voltages across them (a 1 nOhm short beside strips of a
    // few hundred siemens); the mixed-precision solve applies such a preconditioner in FP64
    std::vector<char> stiff;
    // a derived set (gt_operators_derive): the panels and pivots above are its base's; nlow branches beyond the
    // base's are added by the Woodbury identity with W = S^-1 U (node order) and Minv = (Z + U^T W)^-1 per
    // factorisation
    const gt_operators* base = nullptr;
    int nlow = 0;
    int* low_ends = nullptr;     // [2 nlow] dense node index of each added branch's ends
    c64* low_w64 = nullptr;      // [nfact][nlow][nnode]
    c32* low_w32 = nullptr;
    c64* low_m64 = nullptr;      // [nfact][nlow][nlow]
    c32* low_m32 = nullptr;
};

namespace gt {

// the operators' sheet impedances [op][S] and, with face sheets, the face couplings [op][ntw] from the host's
// zs [op][S + ntw]
static void upload_zs(gt_operators* O, const gt_geometry* G, const double* zs, int n_ops, cudaStream_t st = 0) {
    const int S = G->geo.S, ntw = G->ntw, ld = S + ntw;
    std::vector<c64> a((size_t)n_ops * S), b((size_t)n_ops * std::max(ntw, 1));
    for (int q = 0; q < n_ops; ++q) {
        for (int k = 0; k < S; ++k) a[(size_t)q * S + k] = mk<double>(zs[2 * ((size_t)q * ld + k)], zs[2 * ((size_t)q * ld + k) + 1]);
        for (int m = 0; m < ntw; ++m)
            b[(size_t)q * ntw + m] = mk<double>(zs[2 * ((size_t)q * ld + S + m)], zs[2 * ((size_t)q * ld + S + m) + 1]);
    }
    O->zs = O->pool.upload(a.data(), a.size(), st);
    O->zmut = O->pool.upload(b.data(), b.size(), st);
    GT_CUDA(cudaStreamSynchronize(st));      // a and b go out of scope
}

static int status_of(const CudaError& e) {
    set_error(std::string(cudaGetErrorString(e.code)) + " (" + e.where + ")");
    return e.code == cudaErrorMemoryAllocation ? GT_OUT_OF_MEMORY : GT_DEVICE_ERROR;
}

template <typename R> static const R* spec_of(const Orient& o);
template <> const float* spec_of<float>(const Orient& o) { return o.spec32; }
template <> const double* spec_of<double>(const Orient& o) { return o.spec64; }
template <typename R> static const cx<R>* tw0_of(const Orient& o);
template <> const c32* tw0_of<float>(const Orient& o) { return o.tw0_32; }
template <> const c64* tw0_of<double>(const Orient& o) { return o.tw0_64; }
template <typename R> static const cx<R>* tw1_of(const Orient& o);
template <> const c32* tw1_of<float>(const Orient& o) { return o.tw1_32; }
template <> const c64* tw1_of<double>(const Orient& o) { return o.tw1_64; }
template <typename R> static const cx<R>* panel_of(const gt_operators* ops);
template <> const c32* panel_of<float>(const gt_operators* ops) { return ops->panel32; }
template <> const c64* panel_of<double>(const gt_operators* ops) { return ops->panel64; }
template <typename R> static const cx<R>* panel_rm_of(const gt_operators* ops);
template <> const c32* panel_rm_of<float>(const gt_operators* ops) { return ops->panel32_rm; }
template <> const c64* panel_rm_of<double>(const gt_operators* ops) { return ops->panel64_rm; }
template <typename R> static const cx<R>* tab_of(const gt_operators* ops);
template <> const c32* tab_of<float>(const gt_operators* ops) { return ops->tab32; }
template <> const c64* tab_of<double>(const gt_operators* ops) { return ops->tab; }
template <typename R> static const cx<R>* dinv_of(const gt_operators* ops);
template <> const c32* dinv_of<float>(const gt_operators* ops) { return ops->dinv32; }
template <> const c64* dinv_of<double>(const gt_operators* ops) { return ops->dinv64; }
template <typename R> static const cx<R>* low_w_of(const gt_operators* ops);
template <> const c32* low_w_of<float>(const gt_operators* ops) { return ops->low_w32; }
template <> const c64* low_w_of<double>(const gt_operators* ops) { return ops->low_w64; }
template <typename R> static const cx<R>* low_m_of(const gt_operators* ops);
template <> const c32* low_m_of<float>(const gt_operators* ops) { return ops->low_m32; }
template <> const c64* low_m_of<double>(const gt_operators* ops) { return ops->low_m64; }

// A factorisation is stiff when a branch or capacitance admittance of its table exceeds the largest strip
// admittance by more than this: the preconditioner's branch currents D^-1 (r + y_a - y_b) then rest on node
// potential differences below FP32's resolution of the potentials themselves (measured: ratios of 1.6e3 solve
// as usual, 1.6e4 take an extra refinement step, 1.6e6 stall), and the mixed-precision solve applies it in FP64.
constexpr double STIFF_RATIO = 4096.0;

static std::vector<char> stiffness(const std::vector<c64>& t64, int nf, const Geo& g) {
    std::vector<char> out(nf, 0);
    for (int f = 0; f < nf; ++f) {
        const c64* t = t64.data() + (size_t)f * g.ntab;
        double strip = 0, tail = 0;
        for (int e = 0; e < g.tab_cap0; ++e) strip = std::max(strip, std::hypot(t[e].re, t[e].im));
        for (int e = g.tab_cap0; e < g.ntab; ++e) tail = std::max(tail, std::hypot(t[e].re, t[e].im));
        out[f] = strip > 0 && tail > STIFF_RATIO * strip;
    }
    return out;
}

static bool good_fft_size(int P) {
    if (P < 8) return false;
    if (P % 3 == 0) P /= 3;
    return P >= 8 && (P & (P - 1)) == 0;
}

// The FFT passes' launch shapes (rows per row-pass block, columns per column-pass block), chosen once per
// orientation and precision by timing each candidate on the call's own data (two runs each, CUDA events).
template <typename R>
static void tune_lp(Orient& o, LpArgs<R> a, int pr, cudaStream_t st) {
    static const int cand_rows[] = {1, 2, 4, 8, 16};
    static const int cand_bt[] = {1, 2, 4, 8};
    cudaEvent_t e0, e1;
    GT_CUDA(cudaEventCreate(&e0));
    GT_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int br = 4, bb = 2;
    for (int r : cand_rows)
        for (int b : cand_bt) {
            a.rows = r;
            a.bt = b;
            int rr, bb2;
            lp_shapes<R>(a, &rr, &bb2);
            if (rr != r || bb2 != b) continue;   // not a legal shape here
            launch_lp<R>(a, st);
            GT_CUDA(cudaEventRecord(e0, st));
            launch_lp<R>(a, st);
            GT_CUDA(cudaEventRecord(e1, st));
            GT_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            GT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                br = r;
                bb = b;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    o.rows[pr] = br;
    o.bt[pr] = bb;
}

// System product out = K x (mode 0), rhs - K x (1), or the L_p product of the strips (2).
template <typename R>
static void matvec(gt_geometry* G, gt_operators* ops, const cx<R>* x, const cx<R>* rhs, cx<R>* out, int64_t ld, int ncol,
                   const int* col_op, int mode, cx<R>* T, cudaStream_t st, const int* col_list = nullptr) {
    Profiler* P = &G->prof;
    for (int k = 0; k < 2; ++k) {
        Orient& o = G->o[k];
        if ((int64_t)o.n0 * o.n1 == 0) continue;
        LpArgs<R> a{};
        a.x = x;
        a.rhs = rhs;
        a.out = out;
        a.ld = ld;
        a.off = o.off;
        a.off_v = G->geo.off_v;
        a.S = G->geo.S;
        a.n0 = o.n0;
        a.n1 = o.n1;
        a.nx = G->geo.nx;
        a.ny = G->geo.ny;
        a.di = o.di;
        a.dj = o.dj;
        a.P0 = o.P0;
        a.P1 = o.P1;
        a.ncol = ncol;
        a.tw0 = tw0_of<R>(o);
        a.tw1 = tw1_of<R>(o);
        a.spec = spec_of<R>(o);
        a.T = T;
        a.ldt = o.ld0;
        a.mask = G->geo.mask;
        a.col_op = col_op;
        a.omega = ops->omega;
        a.zs = ops->zs;
        a.mode = mode;
        a.col_list = col_list;
        a.sheet_layer = G->geo.NL < G->geo.S ? G->geo.sheet_layer : nullptr;
        const int pr = sizeof(R) == 8;
        if (G->o[k].rows[pr] == 0 && ncol >= 8 && mode != 2) tune_lp<R>(G->o[k], a, pr, st);
        a.rows = o.rows[pr];
        a.bt = o.bt[pr];
        // algorithmic bytes per pass: A reads the strips and writes the intermediate grid; B reads and writes
        // the grid and reads the spectrum once per column group; C reads the grid, the strips and V and
        // writes out
        const double es = sizeof(cx<R>), plane = (double)a.S * o.n0 * o.n1, grid = (double)a.S * o.n0 * o.P1;
        const bool f32 = sizeof(R) == 4;
        {
            Scope s(P, f32 ? "lp_a_f32" : "lp_a_f64", st, ncol * es * (plane + grid));
            launch_lp_pass<R>(a, 0, st);
        }
        {
            Scope s(P, f32 ? "lp_b_f32" : "lp_b_f64", st,
                    ncol * es * 2.0 * grid +
                        std::ceil(ncol / 8.0) * sizeof(R) * a.S * a.S * (o.P0 / 2 + 1) * (o.P1 / 2 + 1));
            launch_lp_pass<R>(a, 1, st);
        }
        {
            Scope s(P, f32 ? "lp_c_f32" : "lp_c_f64", st, ncol * es * (grid + 2.0 * plane));
            launch_lp_pass<R>(a, 2, st);
        }
    }
    if (mode != 2) {
        const double nXY = (double)(G->geo.off_c - G->geo.off_x);
        Scope s(P, sizeof(R) == 4 ? "tail_f32" : "tail_f64", st,
                ncol * (double)sizeof(cx<R>) * (2.0 * (G->geo.n - nXY) + nXY));
        launch_tail<R>(G->geo, x, rhs, out, ld, ncol, col_op, ops->zcap, ops->zbr, mode, col_list, st);
    }
    if (G->narrow.nrow) {
        Scope s(P, "narrow", st);
        launch_narrow<R>(G->narrow, x, out, ld, ncol, G->geo.S, col_op, ops->omega, ops->zs, ops->zmut, mode,
                         col_list, st);
    }
}

// out = M^-1 r for nslot slots whose vectors are ldr apart (inputs) and ldo apart (outputs)
template <typename R>
static void precond(gt_geometry* G, gt_operators* ops, const cx<R>* r, int64_t ldr, cx<R>* out, int64_t ldo, int nslot,
                    const int* slot_op, const Groups& grp, int gmax, cx<R>* zfac, cx<R>* yfac, cx<R>* uvec, cx<R>* sd,
                    cudaStream_t st,
                    const int* col_list = nullptr) {
    Profiler* P = &G->prof;
    if (!panel_of<R>(ops) || !panel_rm_of<R>(ops))
        throw Invalid("these operators keep their FP32 panels only (GT_OPS_FP32_PANELS): no FP64 preconditioner");
    const double es = sizeof(cx<R>), n = (double)G->geo.n, nfac = (double)G->F.nfac;
    const double nodes = (double)G->geo.S * G->geo.nx * G->geo.ny, nXYC = (double)(G->geo.off_b - G->geo.off_x);
    // the factor's panels are read once per column group in each direction
    const double panel = (double)grp.ngroup * es * G->F.panel_total;
    {
        Scope s(P, "pc_node", st, nslot * es * (nXYC + nodes + nfac));
        launch_pc_node<R>(G->geo, r, ldr, yfac, nslot, slot_op, tab_of<R>(ops), col_list, st);
    }
    const cx<R>* pan = panel_of<R>(ops);
    const int nlev = (int)G->level_ptr.size() - 1;
    const int nsub = P->levels ? 1 : std::min(gt_geometry::NSUB, grp.ngroup);
    if (nsub > 1) {
        // forward and backward sweeps per stream, each on a share of the column groups
        Scope s(P, sizeof(R) == 4 ? "fwdbwd_f32" : "fwdbwd_f64", st,
                2 * panel + nslot * es * (4 * nfac + 2.0 * G->F.vec_total));
        G->make_streams();
        GT_CUDA(cudaEventRecord(G->fork, st));
        for (int k = 0; k < nsub; ++k) {
            cudaStream_t sk = G->sub[k];
            GT_CUDA(cudaStreamWaitEvent(sk, G->fork, 0));
            const int g0 = (int)((int64_t)k * grp.ngroup / nsub), g1 = (int)((int64_t)(k + 1) * grp.ngroup / nsub);
            const Groups gk{g1 - g0, grp.gptr + g0, grp.gslot, grp.op + g0};
            for (int h = 0; h < nlev; ++h) {
                const int nf = (int)(G->level_ptr[h + 1] - G->level_ptr[h]);
                launch_fwd_level<R>(G->F, G->d_order + G->level_ptr[h], nf, G->level_maxnf[h], G->level_maxnown[h],
                                    pan, dinv_of<R>(ops), yfac, zfac, uvec, yfac, gk, gmax, sk);
            }
            for (int h = nlev - 1; h >= 0; --h) {
                const int nf = (int)(G->level_ptr[h + 1] - G->level_ptr[h]);
                launch_bwd_level<R>(G->F, G->d_order + G->level_ptr[h], nf, G->level_maxnf[h], G->level_maxnown[h],
                                    panel_rm_of<R>(ops), zfac, yfac, sd, gk, gmax, sk);
            }
            GT_CUDA(cudaEventRecord(G->join[k], sk));
            GT_CUDA(cudaStreamWaitEvent(st, G->join[k], 0));
        }
    } else {
    {
        Scope s(P, sizeof(R) == 4 ? "fwd_f32" : "fwd_f64", st, panel + nslot * es * (2 * nfac + 2.0 * G->F.vec_total));
        for (int h = 0; h < nlev; ++h) {
            int nf = (int)(G->level_ptr[h + 1] - G->level_ptr[h]);
            Scope sl(P->levels ? P : nullptr, (std::string(sizeof(R) == 4 ? "fwd_f32.L" : "fwd_f64.L") +
                                               std::to_string(h)).c_str(), st, grp.ngroup * es * G->level_panel[h]);
            launch_fwd_level<R>(G->F, G->d_order + G->level_ptr[h], nf, G->level_maxnf[h], G->level_maxnown[h], pan,
                                dinv_of<R>(ops), yfac, zfac, uvec, yfac, grp, gmax, st);
        }
    }
    {
        Scope s(P, sizeof(R) == 4 ? "bwd_f32" : "bwd_f64", st, panel + nslot * es * 2 * nfac);
        for (int h = nlev - 1; h >= 0; --h) {
            int nf = (int)(G->level_ptr[h + 1] - G->level_ptr[h]);
            Scope sl(P->levels ? P : nullptr, (std::string(sizeof(R) == 4 ? "bwd_f32.L" : "bwd_f64.L") +
                                               std::to_string(h)).c_str(), st, grp.ngroup * es * G->level_panel[h]);
            launch_bwd_level<R>(G->F, G->d_order + G->level_ptr[h], nf, G->level_maxnf[h], G->level_maxnown[h],
                                panel_rm_of<R>(ops), zfac, yfac, sd, grp, gmax, st);
        }
    }
    }
    if (ops->nlow) {
        // the derived stack's added branches: y -= W Minv U^T y (the coefficients in zfac, free after the sweeps)
        Scope s(P, "lowrank", st, nslot * es * (double)G->F.nnode * (ops->nlow + 2));
        launch_lowrank<R>(sd, G->F.nnode, nslot, ops->nlow, ops->low_ends, low_w_of<R>(ops), low_m_of<R>(ops), slot_op,
                          col_list, zfac, G->F.nfac, st);
    }
    {
        Scope s(P, "pc_strip", st, nslot * es * (2 * n + nfac));
        launch_pc_strip<R>(G->geo, r, ldr, sd, out, ldo, nslot, slot_op, tab_of<R>(ops), col_list, st);
    }
}

// The triangular sweeps stage, per block, a front's rows for every column of a group in shared memory: the own
// and boundary rows of the forward assembly (max_nown + max_nf), the own rows plus up to 17 x 32 rows of tiles
// and partial sums of the forward products (max_nown + 544), the front's rows plus up to 16 x 32 partial sums of
// the backward products (max_nf + 512).  The widest group of 8, 4, 2 or 1 columns whose staging fits a block's
// 227 KB is taken (narrower groups read the panel once per fewer columns); 0 when not even one column fits.
static int group_width(const gt_geometry* G, size_t elem) {
    size_t nown = 1;
    for (int v : G->level_maxnown) nown = std::max(nown, (size_t)v);
    const size_t nf = (size_t)std::max(G->max_nf, 1);
    const size_t rows = std::max({nown + nf, nown + 544, nf + 512});
    const char* cap_env = std::getenv("GT_GROUP_WIDTH");       // a lower cap, for tests of the narrow groups
    const int cap = cap_env ? std::atoi(cap_env) : 8;
    for (int gc : {8, 4, 2, 1})
        if (gc <= cap && (size_t)gc * rows * elem <= 227 * 1024) return gc;
    return 0;
}

static bool solve_fits(const gt_geometry* G, size_t elem) { return group_width(G, elem) > 0; }

static int group_max(const gt_geometry* G, size_t elem) {
    const int gc = group_width(G, elem);
    if (!gc) throw Invalid("a front is too large for the triangular-solve kernels' shared memory");
    return gc;
}


// the listed slots (sorted by operator) -> groups of <= gmax slots sharing one operator:
// group g holds gslot[gptr[g] .. gptr[g+1])
static void make_groups(const std::vector<int>& slots, const std::vector<int>& slot_op, int gmax, std::vector<int>& gptr,
                        std::vector<int>& gslot, std::vector<int>& op) {
    gptr.assign(1, 0);
    gslot.clear();
    op.clear();
    int n = (int)slots.size();
    for (int s = 0; s < n;) {
        int e = s;
        while (e < n && slot_op[slots[e]] == slot_op[slots[s]] && e - s < gmax) ++e;
        for (int q = s; q < e; ++q) gslot.push_back(slots[q]);
        gptr.push_back((int)gslot.size());
        op.push_back(slot_op[slots[s]]);
        s = e;
    }
}

// W = S^-1 U for a derived operator set: the base's sweeps (precision R) on U e_j, column c = f k + j of
// the nf factorisations' k added branches, in batches; w: [nf k][nnode] node order
template <typename R>
static void lowrank_w(gt_geometry* G, const gt_operators* base, int nf, int k, const int* ends, cx<R>* w,
                      cudaStream_t st) {
    const int64_t nnode = G->F.nnode, nfac = G->F.nfac, ntot = (int64_t)nf * k;
    const int gmax = group_max(G, sizeof(cx<R>));
    const int bc = (int)std::min<int64_t>(ntot, 64);
    Pool tmp;
    cx<R>* sv = tmp.alloc<cx<R>>((size_t)bc * nfac);
    cx<R>* zv = tmp.alloc<cx<R>>((size_t)bc * nfac);
    cx<R>* uv = tmp.alloc<cx<R>>((size_t)bc * std::max<int64_t>(G->F.vec_total, 1));
    int* d_gptr = tmp.alloc<int>(bc + 1);
    int* d_gslot = tmp.alloc<int>(bc);
    int* d_gop = tmp.alloc<int>(bc);
    const int nlev = (int)G->level_ptr.size() - 1;
    for (int64_t c0 = 0; c0 < ntot; c0 += bc) {
        const int nc = (int)std::min<int64_t>(bc, ntot - c0);
        cx<R>* wout = w + c0 * nnode;
        GT_CUDA(cudaMemsetAsync(sv, 0, (size_t)nc * nfac * sizeof(cx<R>), st));
        GT_CUDA(cudaMemsetAsync(wout, 0, (size_t)nc * nnode * sizeof(cx<R>), st));
        launch_lowrank_rhs<R>(sv, nfac, (int)c0, nc, k, ends, G->geo.perm, st);
        std::vector<int> slots(nc), sfact(nc), gptr, gslot, gop;
        for (int q = 0; q < nc; ++q) {
            slots[q] = q;
            sfact[q] = (int)((c0 + q) / k);
        }
        make_groups(slots, sfact, gmax, gptr, gslot, gop);
        GT_CUDA(cudaMemcpy(d_gptr, gptr.data(), gptr.size() * sizeof(int), cudaMemcpyHostToDevice));
        GT_CUDA(cudaMemcpy(d_gslot, gslot.data(), gslot.size() * sizeof(int), cudaMemcpyHostToDevice));
        GT_CUDA(cudaMemcpy(d_gop, gop.data(), gop.size() * sizeof(int), cudaMemcpyHostToDevice));
        const Groups grp{(int)gop.size(), d_gptr, d_gslot, d_gop};
        for (int h = 0; h < nlev; ++h) {
            const int nfl = (int)(G->level_ptr[h + 1] - G->level_ptr[h]);
            launch_fwd_level<R>(G->F, G->d_order + G->level_ptr[h], nfl, G->level_maxnf[h], G->level_maxnown[h],
                                panel_of<R>(base), dinv_of<R>(base), sv, zv, uv, sv, grp, gmax, st);
        }
        for (int h = nlev - 1; h >= 0; --h) {
            const int nfl = (int)(G->level_ptr[h + 1] - G->level_ptr[h]);
            launch_bwd_level<R>(G->F, G->d_order + G->level_ptr[h], nfl, G->level_maxnf[h], G->level_maxnown[h],
                                panel_rm_of<R>(base), zv, sv, wout, grp, gmax, st);
        }
        GT_CUDA(cudaStreamSynchronize(st));   // the group tables are reused by the next batch
    }
}

static int nchunks(int64_t n) { return (int)((n + 2047) / 2048); }  // DOT_CHUNK in gmres.cu

static void fill_ws(Workspace& W, gt_geometry* G, int ncol, int m, int prec, int kmax, cudaStream_t st);

// The solve workspace for ncol columns, made on first use; its clears are ordered on the solve's stream st.
static void ensure_ws(gt_geometry* G, int ncol, int m, int prec, int kmax, cudaStream_t st) {
    auto& w = G->ws;
    if (w && w->ncol >= ncol && w->m >= m && w->prec == prec && w->kmax >= kmax) return;
    if (w) {                       // the old one's last kernels are done before its memory goes
        cudaDeviceSynchronize();
        w.reset();
    }
    w.reset(new Workspace());
    fill_ws(*w, G, ncol, m, prec, kmax, st);
}

// the bytes fill_ws would allocate (nothing is allocated)
static size_t ws_bytes(gt_geometry* G, int ncol, int m, int prec, int kmax) {
    Workspace W;
    W.pool.dry = true;
    fill_ws(W, G, ncol, m, prec, kmax, 0);
    return W.pool.bytes;
}

static void fill_ws(Workspace& W, gt_geometry* G, int ncol, int m, int prec, int kmax, cudaStream_t st) {
    const bool dry = W.pool.dry;
    W.ncol = ncol;
    W.m = m;
    W.prec = prec;
    W.kmax = kmax;
    const int64_t n = G->geo.n;
    const size_t es = prec == 1 ? sizeof(c64) : sizeof(c32);
    const size_t eb = prec == 2 ? sizeof(h16c) : es;     // basis entries
    Pool& p = W.pool;
    W.x64 = p.alloc<c64>((size_t)ncol * n);
    W.r64 = p.alloc<c64>((size_t)ncol * n);
    W.b64 = p.alloc<c64>((size_t)ncol * n);
    W.T64 = p.alloc<c64>((size_t)ncol * G->maxT);
    W.rho = p.alloc<double>(ncol);
    W.bnorm = p.alloc<double>(ncol);
    const int nch = nchunks(n);
    W.npart = p.alloc<c64>((size_t)ncol * std::max(nch, update_chunks(n)));
    W.npart_k = p.alloc<c64>((size_t)ncol * nch * (kmax + 2));
    W.nred = p.alloc<c64>(ncol);
    W.V = p.alloc<unsigned char>((size_t)ncol * (m + 1) * n * eb);
    if (prec == 2) W.vcur = p.alloc<unsigned char>((size_t)ncol * n * es);
    W.w = p.alloc<unsigned char>((size_t)ncol * n * es);
    W.z = p.alloc<unsigned char>((size_t)ncol * n * es);
    W.T = p.alloc<unsigned char>((size_t)ncol * G->maxT * es);
    W.zfac = p.alloc<unsigned char>((size_t)ncol * G->F.nfac * es);
    W.yfac = p.alloc<unsigned char>((size_t)ncol * G->F.nfac * es);
    W.uvec = p.alloc<unsigned char>((size_t)ncol * std::max<int64_t>(G->F.vec_total, 1) * es);
    // node-ordered s / y of the preconditioner: entries of nodes that are not kept stay zero
    W.sd = p.alloc<unsigned char>((size_t)ncol * G->F.nnode * es);
    if (!dry) GT_CUDA(cudaMemsetAsync(W.sd, 0, (size_t)ncol * G->F.nnode * es, st));
    W.partial = p.alloc<c64>((size_t)ncol * nch * (m + 2));
    if (prec == 3) {
        W.pr64 = p.alloc<c64>((size_t)ncol * n);
        W.pz64 = p.alloc<c64>((size_t)ncol * n);
        W.zfac64 = p.alloc<c64>((size_t)ncol * G->F.nfac);
        W.yfac64 = p.alloc<c64>((size_t)ncol * G->F.nfac);
        W.uvec64 = p.alloc<c64>((size_t)ncol * std::max<int64_t>(G->F.vec_total, 1));
        W.sd64 = p.alloc<c64>((size_t)ncol * G->F.nnode);
        if (!dry) GT_CUDA(cudaMemsetAsync(W.sd64, 0, (size_t)ncol * G->F.nnode * sizeof(c64), st));
    }
    GmresState& s = W.st;
    s.nslot = ncol;
    s.m = m;
    s.ldh = m + 2;
    s.H = p.alloc<c64>((size_t)ncol * (m + 1) * m);
    s.cs = p.alloc<double>((size_t)ncol * m);
    s.sn = p.alloc<c64>((size_t)ncol * m);
    s.g = p.alloc<c64>((size_t)ncol * (m + 1));
    s.hvec = p.alloc<c64>((size_t)ncol * s.ldh);
    s.h2vec = p.alloc<c64>((size_t)ncol * s.ldh);
    s.y = p.alloc<c64>((size_t)ncol * s.ldh);
    s.hn2 = p.alloc<c64>(ncol);
    s.hn2b = p.alloc<c64>(ncol);
    s.it = p.alloc<int>(ncol);
    s.its_total = p.alloc<int>(ncol);
    s.active = p.alloc<int>(ncol);
    s.reorth = p.alloc<int>(ncol);
    s.eta = p.alloc<double>(ncol);
    s.inv_hn = p.alloc<double>(ncol);
    s.resid_est = p.alloc<double>(ncol);
    W.slot_col = p.alloc<int>(ncol);
    W.slot_op = p.alloc<int>(ncol);
    W.slot_pc = p.alloc<int>(ncol);
    W.g_ptr = p.alloc<int>(ncol + 1);
    W.g_slot = p.alloc<int>(ncol);
    W.g_op = p.alloc<int>(ncol);
    W.act = p.alloc<int>(ncol);
    if (!dry) GT_CUDA(cudaMallocHost(&W.act_host, ncol * sizeof(int)));
    W.gP = p.alloc<c64>((size_t)kmax * ncol * n);
    W.gQ = p.alloc<c64>((size_t)kmax * ncol * n);
    W.gbeta = p.alloc<c64>((size_t)ncol * (kmax + 1));
    W.galpha = p.alloc<c64>((size_t)ncol * 2);
    W.gnu2 = p.alloc<c64>(ncol);
    W.colact = p.alloc<int>(ncol);
    W.col_op = p.alloc<int>(ncol);
    W.flag_dev = p.alloc<int>(1);
    W.its_col = p.alloc<int>(ncol);
    if (dry) return;
    GT_CUDA(cudaMallocHost(&W.flag_host, sizeof(int)));
    GT_CUDA(cudaMemsetAsync(W.V, 0, (size_t)ncol * (m + 1) * n * eb, st));
}

// ||v_c|| for ncol FP64 dense vectors -> out (device)
static void norms64(gt_geometry* G, const c64* v, int64_t ld, int ncol, double* out, cudaStream_t st) {
    Workspace& W = *G->ws;
    const int nch = nchunks(G->geo.n);
    launch_dots<double>(v, 0, ld, 0, v, ld, G->geo.n, ncol, nullptr, W.npart, nch, st);
    launch_reduce(W.npart, nch, 0, ncol, nullptr, W.nred, 1, 0, st);
    launch_sqrt_norms(W.nred, 1, ncol, out, st);
}

// R: the inner GMRES arithmetic; B: its basis storage (cx<R>, or FP16 pairs scaled by a power of two near
// sqrt(n) so that a unit vector's entries sit near 1)
template <typename R, typename B = cx<R>>
static int solve_impl(gt_geometry* G, gt_operators* ops, int ncol, const int* h_col_op, const gt_solve_opts& o,
                      int* its_out, double* resid_out, cudaStream_t st, bool pc64 = false) {
    constexpr bool narrow = !std::is_same<B, cx<R>>::value;
    Workspace& W = *G->ws;
    const int64_t n = G->geo.n;
    const int m = o.restart;
    const int nch = nchunks(n), nchu = update_chunks(n);
    Profiler* P = &G->prof;
    GT_CUDA(cudaMemcpyAsync(W.col_op, h_col_op, ncol * sizeof(int), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaMemsetAsync(W.its_col, 0, ncol * sizeof(int), st));
    norms64(G, W.b64, n, ncol, W.bnorm, st);
    if (o.use_guess) {
        // x holds the starting points: r = b - K x in FP64
        matvec<double>(G, ops, W.x64, W.b64, W.r64, n, ncol, W.col_op, 1, W.T64, st);
        norms64(G, W.r64, n, ncol, W.rho, st);
    } else {
        GT_CUDA(cudaMemsetAsync(W.x64, 0, (size_t)ncol * n * sizeof(c64), st));
        GT_CUDA(cudaMemcpyAsync(W.r64, W.b64, (size_t)ncol * n * sizeof(c64), cudaMemcpyDeviceToDevice, st));
        GT_CUDA(cudaMemcpyAsync(W.rho, W.bnorm, ncol * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    std::vector<double> h_bnorm(ncol), h_rho(ncol);
    std::vector<int> h_its(ncol, 0);
    GT_CUDA(cudaMemcpyAsync(h_bnorm.data(), W.bnorm, ncol * sizeof(double), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaMemcpyAsync(h_rho.data(), W.rho, ncol * sizeof(double), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    const int gmax = group_max(G, pc64 ? sizeof(c64) : sizeof(cx<R>));
    B* V = static_cast<B*>(W.V);
    cx<R>* vcur = narrow ? static_cast<cx<R>*>(W.vcur) : nullptr;
    const R bscale = narrow ? R(std::ldexp(1.0, (int)std::lround(0.5 * std::log2((double)n)))) : R(1);
    const R vs = R(1) / bscale;
    cx<R>* w = static_cast<cx<R>*>(W.w);
    cx<R>* z = static_cast<cx<R>*>(W.z);
    cx<R>* T = static_cast<cx<R>*>(W.T);
    cx<R>* zfac = static_cast<cx<R>*>(W.zfac);
    cx<R>* yfac = static_cast<cx<R>*>(W.yfac);
    cx<R>* uvec = static_cast<cx<R>*>(W.uvec);
    cx<R>* sd = static_cast<cx<R>*>(W.sd);
    const int64_t lds = (int64_t)(m + 1) * n;
    // the preconditioner on nsl listed slots (outputs n apart): in precision R, or, for stiff factorisations
    // (pc64), in FP64 on FP64 copies of the vectors, its result rounded back to R
    auto apply_pc = [&](const cx<R>* rin, int64_t ldr, cx<R>* out, int nsl, const Groups& g, const int* list) {
        if constexpr (std::is_same<R, float>::value) {
            if (pc64) {
                launch_recast<double, float>(W.pr64, n, rin, ldr, list, n, nsl, st);
                precond<double>(G, ops, W.pr64, n, W.pz64, n, nsl, W.slot_pc, g, gmax, W.zfac64, W.yfac64, W.uvec64,
                                W.sd64, st, list);
                launch_recast<float, double>(out, n, W.pz64, n, list, n, nsl, st);
                return;
            }
        }
        precond<R>(G, ops, rin, ldr, out, n, nsl, W.slot_pc, g, gmax, zfac, yfac, uvec, sd, st, list);
    };
    std::vector<int> slot_col, slot_op, slot_pc, gptr, gslot, gop, act;
    auto upload_groups = [&](const std::vector<int>& slots) {
        make_groups(slots, slot_pc, gmax, gptr, gslot, gop);
        GT_CUDA(cudaMemcpyAsync(W.act, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        GT_CUDA(cudaMemcpyAsync(W.g_ptr, gptr.data(), gptr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        GT_CUDA(cudaMemcpyAsync(W.g_slot, gslot.data(), gslot.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        GT_CUDA(cudaMemcpyAsync(W.g_op, gop.data(), gop.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        return Groups{(int)gop.size(), W.g_ptr, W.g_slot, W.g_op};
    };
    const int K = std::max(1, o.outer_k);
    const int64_t ldk = (int64_t)ncol * n;          // between GCR directions
    int k = 0;                                      // directions held
    bool verified = true;                           // rho is the true residual's norm
    std::vector<int> colact(ncol);
    // the true residual r = b - K x in FP64 (and its norms), which also restarts the GCR directions
    auto true_residual = [&]() {
        matvec<double>(G, ops, W.x64, W.b64, W.r64, n, ncol, W.col_op, 1, W.T64, st);
        {
            Scope sc(P, "norms", st, 16.0 * ncol * n);
            norms64(G, W.r64, n, ncol, W.rho, st);
        }
        GT_CUDA(cudaMemcpyAsync(h_rho.data(), W.rho, ncol * sizeof(double), cudaMemcpyDeviceToHost, st));
        GT_CUDA(cudaStreamSynchronize(st));
        verified = true;
        k = 0;
    };
    for (int outer = 0; outer < o.max_outer; ++outer) {
        auto pick = [&]() {
            slot_col.clear();
            for (int c = 0; c < ncol; ++c)
                if (h_bnorm[c] > 0 && h_rho[c] > o.tol * h_bnorm[c] && h_its[c] < o.max_its) slot_col.push_back(c);
        };
        pick();
        if (slot_col.empty() && !verified) {        // the recurrence says done: confirm on the true residual
            true_residual();
            pick();
        }
        if (slot_col.empty()) break;
        // slots sorted by factorisation, then operator: the columns sharing a factor read it together
        std::stable_sort(slot_col.begin(), slot_col.end(), [&](int a, int b) {
            const int fa = ops->fslot[h_col_op[a]], fb = ops->fslot[h_col_op[b]];
            return fa != fb ? fa < fb : h_col_op[a] < h_col_op[b];
        });
        const int ns = (int)slot_col.size();
        slot_op.resize(ns);
        slot_pc.resize(ns);
        for (int s = 0; s < ns; ++s) {
            slot_op[s] = h_col_op[slot_col[s]];
            slot_pc[s] = ops->fslot[slot_op[s]];
        }
        GT_CUDA(cudaMemcpyAsync(W.slot_col, slot_col.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
        GT_CUDA(cudaMemcpyAsync(W.slot_op, slot_op.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
        GT_CUDA(cudaMemcpyAsync(W.slot_pc, slot_pc.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
        act.resize(ns);
        for (int q = 0; q < ns; ++q) act[q] = q;
        std::vector<int> its_slot(ns);
        for (int s = 0; s < ns; ++s) its_slot[s] = h_its[slot_col[s]];
        GmresState S = W.st;
        S.nslot = ns;
        S.m = m;
        S.max_its = o.max_its;
        S.reorth_ratio = o.reorth;
        GT_CUDA(cudaMemcpyAsync(S.its_total, its_slot.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
        Groups grp = upload_groups(act);
        GmresStateT<R, B> ST{ns, S.active, S.inv_hn, V, w, n, lds, bscale, vcur};
        {
            Scope sc(P, "gmres_small", st);
            launch_init_state(S, W.slot_col, W.rho, W.bnorm, o.tol, o.inner_tol, st);
            launch_init_cycle<R, B>(ST, W.r64, n, W.slot_col, W.rho, n, st);
        }
        int jdone = 0;
        for (int j = 0; j < m; ++j) {
            // the products run on the slots still iterating in this cycle (W.act, grp)
            const int na = (int)act.size();
            // the product is applied to the basis vector as stored
            const cx<R>* vin;
            int64_t ldin;
            if constexpr (narrow) {
                vin = vcur;
                ldin = n;
            } else {
                vin = V + (int64_t)j * n;
                ldin = lds;
            }
            apply_pc(vin, ldin, z, na, grp, W.act);
            matvec<R>(G, ops, z, nullptr, w, n, na, W.slot_op, 0, T, st, W.act);
            // classical Gram-Schmidt: the dot products read the j+1 basis vectors and w; the update reads
            // them again, reads w and writes it
            {
                Scope sc(P, narrow ? "gs_dots_f32_b16" : sizeof(R) == 4 ? "gs_dots_f32" : "gs_dots_f64", st,
                         (double)ns * n * ((j + 1.0) * sizeof(B) + sizeof(cx<R>)));
                launch_dots<R, B>(V, n, lds, j + 1, w, n, n, ns, S.active, W.partial, nch, st, vs);
                launch_reduce(W.partial, nch, j + 1, ns, S.active, S.hvec, S.ldh, 0, st);
            }
            {
                Scope sc(P, narrow ? "gs_update_f32_b16" : sizeof(R) == 4 ? "gs_update_f32" : "gs_update_f64", st,
                         (double)ns * n * ((j + 1.0) * sizeof(B) + 2.0 * sizeof(cx<R>)));
                launch_update<R, B>(V, n, lds, j + 1, S.hvec, S.ldh, w, n, n, ns, S.active, W.partial, -1, st, vs);
                launch_reduce(W.partial, nchu, 0, ns, S.active, S.hn2, 1, 0, st);
                launch_dgks(S, j, st);
            }
            if (o.reorth > 0) {         // DGKS second pass (the slots launch_dgks flagged)
                Scope sc(P, "gs_reorth", st);
                launch_dots<R, B>(V, n, lds, j + 1, w, n, n, ns, S.reorth, W.partial, nch, st, vs);
                launch_reduce(W.partial, nch, j + 1, ns, S.reorth, S.h2vec, S.ldh, 0, st);
                launch_update<R, B>(V, n, lds, j + 1, S.h2vec, S.ldh, w, n, n, ns, S.reorth, W.partial, -1, st, vs);
                launch_reduce(W.partial, nchu, 0, ns, S.reorth, S.hn2b, 1, 0, st);
            }
            {
                Scope sc(P, "gmres_small", st);
                launch_givens(S, j, st);
                if (j + 1 < m) launch_scale<R, B>(ST, j, n, st);
            }
            GT_CUDA(cudaMemcpyAsync(W.act_host, S.active, ns * sizeof(int), cudaMemcpyDeviceToHost, st));
            GT_CUDA(cudaStreamSynchronize(st));
            jdone = j + 1;
            std::vector<int> still;
            for (int q : act)
                if (W.act_host[q]) still.push_back(q);
            if (still.empty()) break;
            if (still.size() < act.size()) {
                act.swap(still);
                grp = upload_groups(act);
            }
        }
        // the cycle's correction: x += rho * M^-1 (V y)
        {
            Scope sc(P, "gmres_small", st);
            launch_hsolve(S, st);
        }
        GT_CUDA(cudaMemsetAsync(w, 0, (size_t)ns * n * sizeof(cx<R>), st));
        {
            Scope sc(P, "combine", st, (double)ns * n * (jdone * sizeof(B) + 2.0 * sizeof(cx<R>)));
            launch_update<R, B>(V, n, lds, jdone, S.y, S.ldh, w, n, n, ns, nullptr, nullptr, 1, st, vs);
        }
        act.resize(ns);
        for (int q = 0; q < ns; ++q) act[q] = q;
        grp = upload_groups(act);
        apply_pc(w, n, z, ns, grp, W.act);
        // GCR step in FP64: p = the cycle's correction, q = K p, both orthogonalised against the directions
        // held (q orthonormal); then x += alpha p, r -= alpha q with alpha = q^H r
        if (k == K) k = 0;
        c64* Pk = W.gP + (int64_t)k * ldk;
        c64* Qk = W.gQ + (int64_t)k * ldk;
        std::fill(colact.begin(), colact.end(), 0);
        for (int c : slot_col) colact[c] = 1;
        GT_CUDA(cudaMemcpyAsync(W.colact, colact.data(), ncol * sizeof(int), cudaMemcpyHostToDevice, st));
        {
            Scope sc(P, "gcr", st, (double)ns * n * (16.0 * (4 * k + 12) + sizeof(cx<R>)));
            GT_CUDA(cudaMemsetAsync(Pk, 0, (size_t)ldk * sizeof(c64), st));
            launch_to64<R>(Pk, n, z, n, W.slot_col, n, ns, st);
        }
        matvec<double>(G, ops, Pk, nullptr, Qk, n, ns, W.col_op, 0, W.T64, st, W.slot_col);
        {
            Scope sc(P, "gcr", st, 0.0);
            if (k > 0) {
                launch_dots<double>(W.gQ, ldk, n, k, Qk, n, n, ncol, W.colact, W.npart_k, nch, st);
                launch_reduce(W.npart_k, nch, k, ncol, W.colact, W.gbeta, K + 1, 0, st);
                launch_update<double>(W.gQ, ldk, n, k, W.gbeta, K + 1, Qk, n, n, ncol, W.colact, W.npart, -1, st);
                launch_update<double>(W.gP, ldk, n, k, W.gbeta, K + 1, Pk, n, n, ncol, W.colact, nullptr, -1, st);
                launch_reduce(W.npart, nchu, 0, ncol, W.colact, W.gnu2, 1, 0, st);
            } else {
                launch_dots<double>(Qk, 0, n, 0, Qk, n, n, ncol, W.colact, W.npart, nch, st);
                launch_reduce(W.npart, nch, 0, ncol, W.colact, W.gnu2, 1, 0, st);
            }
            launch_gcr_scale(Pk, Qk, n, W.gnu2, W.colact, n, ncol, st);
            launch_dots<double>(Qk, 0, n, 1, W.r64, n, n, ncol, W.colact, W.npart_k, nch, st);
            launch_reduce(W.npart_k, nch, 1, ncol, W.colact, W.galpha, 2, 0, st);
            launch_update<double>(Pk, 0, n, 1, W.galpha, 2, W.x64, n, n, ncol, W.colact, nullptr, 1, st);
            launch_update<double>(Qk, 0, n, 1, W.galpha, 2, W.r64, n, n, ncol, W.colact, W.npart, -1, st);
            launch_reduce(W.npart, nchu, 0, ncol, W.colact, W.nred, 1, 0, st);
            launch_sqrt_norms_active(W.nred, 1, ncol, W.colact, W.rho, st);
        }
        ++k;
        verified = false;
        GT_CUDA(cudaMemcpyAsync(h_rho.data(), W.rho, ncol * sizeof(double), cudaMemcpyDeviceToHost, st));
        GT_CUDA(cudaMemcpyAsync(its_slot.data(), S.its_total, ns * sizeof(int), cudaMemcpyDeviceToHost, st));
        GT_CUDA(cudaStreamSynchronize(st));
        for (int s = 0; s < ns; ++s) h_its[slot_col[s]] = its_slot[s];
        P->flush(st);
    }
    if (!verified) true_residual();
    P->flush(st);
    bool all = true;
    for (int c = 0; c < ncol; ++c) {
        double rr = h_bnorm[c] > 0 ? h_rho[c] / h_bnorm[c] : 0.0;
        if (its_out) its_out[c] = h_its[c];
        if (resid_out) resid_out[c] = rr;
        if (!(rr <= o.tol)) all = false;
    }
    return all ? GT_OK : GT_NOT_CONVERGED;
}

static int run_solve(gt_geometry* G, gt_operators* ops, int ncol, const int* col_op, const gt_solve_opts* opts,
                     int* its, double* res, cudaStream_t st) {
    gt_solve_opts o = *opts;
    if (o.restart < 1 || o.restart > 250) throw Invalid("restart must be in 1..250");
    if (o.max_outer < 1) o.max_outer = 1;
    for (int c = 0; c < ncol; ++c)
        if (col_op[c] < 0 || col_op[c] >= ops->nops) throw Invalid("column operator index out of range");
    if ((o.precision == 1 || o.precision == 3) && (!ops->panel64 || !ops->panel64_rm))
        throw Invalid("precision 1 and 3 need the FP64 panels these operators did not keep (GT_OPS_FP32_PANELS)");
    if (o.precision == 1) return solve_impl<double>(G, ops, ncol, col_op, o, its, res, st);
    if (o.precision == 2) return solve_impl<float, h16c>(G, ops, ncol, col_op, o, its, res, st);
    if (o.precision == 3) {
        if (!solve_fits(G, sizeof(c64))) throw Invalid("precision 3: a front is too large for the FP64 sweeps");
        return solve_impl<float>(G, ops, ncol, col_op, o, its, res, st, true);
    }
    if (o.precision != 0) throw Invalid("precision must be 0, 1, 2 or 3");
    return solve_impl<float>(G, ops, ncol, col_op, o, its, res, st);
}

// precision 0 becomes 3 when a column's factorisation is stiff and the FP64 sweeps fit its fronts
static int effective_precision(const gt_geometry* G, const gt_operators* ops, int ncol, const int* col_op, int prec) {
    if (prec != 0 || !ops || !col_op || ops->stiff.empty() || !solve_fits(G, sizeof(c64))) return prec;
    for (int c = 0; c < ncol; ++c) {
        const int q = col_op[c];
        if (q >= 0 && q < ops->nops && ops->stiff[ops->fslot[q]]) return 3;
    }
    return 0;
}

// The L_p product of n_cols dense FP64 vectors into the strip segments of y, with the FFT passes'
// intermediate grid in caller-provided scratch (used by gt_lp_product_noalloc, noalloc.cu).  Launches
// kernels only: no allocation, no synchronisation.
size_t lp_scratch_bytes(const gt_geometry* G, int ncol) { return (size_t)ncol * (size_t)G->maxT * sizeof(c64); }
int geometry_device(const gt_geometry* G) { return G->device; }

void lp_with_scratch(gt_geometry* G, int ncol, const c64* x, c64* y, void* scratch, cudaStream_t st) {
    for (int k = 0; k < 2; ++k) {
        const Orient& o = G->o[k];
        if ((int64_t)o.n0 * o.n1 == 0) continue;
        LpArgs<double> a{};
        a.x = x;
        a.out = y;
        a.ld = G->geo.n;
        a.off = o.off;
        a.off_v = G->geo.off_v;
        a.S = G->geo.S;
        a.n0 = o.n0;
        a.n1 = o.n1;
        a.nx = G->geo.nx;
        a.ny = G->geo.ny;
        a.di = o.di;
        a.dj = o.dj;
        a.P0 = o.P0;
        a.P1 = o.P1;
        a.ncol = ncol;
        a.tw0 = o.tw0_64;
        a.tw1 = o.tw1_64;
        a.spec = o.spec64;
        a.T = static_cast<c64*>(scratch);
        a.ldt = o.ld0;
        a.mask = G->geo.mask;
        a.mode = 2;
        launch_lp<double>(a, st);
    }
    if (G->narrow.nrow)
        launch_narrow<double>(G->narrow, x, y, G->geo.n, ncol, G->geo.S, nullptr, nullptr, nullptr, nullptr, 2,
                              nullptr, st);
}

}  // namespace gt

// ------------------------------------------------------------------------------------------ C ABI
#define GT_GUARD_BEGIN try {
#define GT_GUARD_END                                                 \
    }                                                                \
    catch (const gt::CudaError& e) {                                 \
        return gt::status_of(e);                                     \
    }                                                                \
    catch (const gt::Invalid& e) {                                   \
        gt::set_error(e.what());                                     \
        return GT_INVALID_ARGUMENT;                                  \
    }                                                                \
    catch (const gt::Timeout& e) {                                   \
        gt::set_error(e.what());                                     \
        return GT_TIMEOUT;                                           \
    }                                                                \
    catch (const std::bad_alloc&) {                                  \
        gt::set_error("host allocation failed");                     \
        return GT_OUT_OF_MEMORY;                                     \
    }                                                                \
    catch (const std::exception& e) {                                \
        gt::set_error(e.what());                                     \
        return GT_DEVICE_ERROR;                                      \
    }

extern "C" {

int gt_version(void) { return 100; }

int64_t gt_launch_count(void) { return gt::g_launches.load(); }

const char* gt_last_error(void) { return gt::t_last_error.c_str(); }

int gt_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int gt_geometry_create(const gt_geometry_desc* d, gt_geometry** out) {
    GT_GUARD_BEGIN
    if (!d || !out) throw Invalid("null argument");
    if (d->n_sheets < 1 || d->n_sheets > 6) throw Invalid("1 to 6 sheets are supported");
    if (d->nx < 3 || d->ny < 3) throw Invalid("grid must be at least 3 x 3");
    for (int k = 0; k < 4; ++k)
        if (!good_fft_size(d->fft_p[k])) throw Invalid("FFT sizes must be 2^a or 3*2^a with a >= 3");
    std::unique_ptr<gt_geometry> G(new gt_geometry());
    Pool& p = G->pool;
    Geo& g = G->geo;
    const int S = d->n_sheets, nx = d->nx, ny = d->ny;
    const int NL = d->n_layers > 0 ? d->n_layers : S;
    if (NL > S || (NL < S && !d->sheet_layer)) throw Invalid("n_layers must not exceed n_sheets; sheet_layer needed");
    const int64_t nn = (int64_t)NL * nx * ny;
    g.S = S;
    g.NL = NL;
    {
        std::vector<int> sl(S);
        for (int k = 0; k < S; ++k) {
            sl[k] = d->sheet_layer && NL < S ? d->sheet_layer[k] : k;
            if (sl[k] < 0 || sl[k] >= NL) throw Invalid("sheet_layer out of range");
        }
        g.sheet_layer = p.upload(sl.data(), sl.size());
    }
    if (d->n_twins < 0 || d->n_twins != S - NL) throw Invalid("n_twins must be n_sheets - n_layers");
    G->ntw = d->n_twins;
    g.nx = nx;
    g.ny = ny;
    g.np = d->n_pairs;
    g.nbr = d->n_branches;
    g.sheet = d->precond_sheet;
    g.n = d->n_dense;
    g.off_x = d->off_x;
    g.off_y = d->off_y;
    g.off_c = d->off_c;
    g.off_b = d->off_b;
    g.off_v = d->off_v;
    g.mask = p.upload(d->mask, d->n_dense);
    g.code_x = p.upload(d->code_x, (size_t)(nx - 1) * ny);
    g.code_y = p.upload(d->code_y, (size_t)nx * (ny - 1));
    g.pair_layers = p.upload(d->pair_layers, (size_t)2 * d->n_pairs);
    g.branch_nodes = p.upload(d->branch_nodes, (size_t)2 * d->n_branches);
    // branch ends per node (CSR over dense nodes)
    std::vector<int> cnt(nn + 1, 0);
    for (int b = 0; b < d->n_branches; ++b)
        for (int e = 0; e < 2; ++e) {
            int node = d->branch_nodes[2 * b + e];
            if (node < 0 || node >= nn) throw Invalid("branch node out of range");
            cnt[node + 1]++;
        }
    for (int64_t i = 0; i < nn; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> idx(std::max(cnt[nn], 1)), fill(cnt.begin(), cnt.end() - 1);
    for (int b = 0; b < d->n_branches; ++b) {
        idx[fill[d->branch_nodes[2 * b]]++] = b + 1;
        idx[fill[d->branch_nodes[2 * b + 1]]++] = -(b + 1);
    }
    g.node_br_ptr = p.upload(cnt.data(), cnt.size());
    g.node_br_idx = p.upload(idx.data(), idx.size());
    g.perm = p.upload(d->perm, nn);
    g.nfac = d->n_factor;
    g.ntab = d->n_table;
    if (d->n_override < 0) throw Invalid("n_override must not be negative");
    g.tab_ovr0 = 2 * (1 << S) * S * S;
    g.tab_cap0 = g.tab_ovr0 + d->n_override * S * S;
    g.tab_br0 = g.tab_cap0 + d->n_pairs;
    if (g.tab_br0 + d->n_branches != d->n_table) throw Invalid("admittance table length mismatch");
    g.cap_fill = nullptr;
    if (d->cap_fill && d->n_pairs > 0) {
        const size_t nc = (size_t)d->n_pairs * nx * ny;
        for (size_t q = 0; q < nc; ++q)
            if (d->mask[d->off_c + (int64_t)q] && !(d->cap_fill[q] > 0.0 && d->cap_fill[q] <= 1.0))
                throw Invalid("cap_fill must be in (0, 1] at every capacitance cell");
        g.cap_fill = p.upload(d->cap_fill, nc);
    }
    g.ovr_x = g.ovr_y = nullptr;
    if (d->n_override > 0) {
        if (!d->override_x || !d->override_y) throw Invalid("override positions missing");
        for (size_t q = 0; q < (size_t)(nx - 1) * ny; ++q)
            if (d->override_x[q] >= d->n_override) throw Invalid("override index out of range");
        for (size_t q = 0; q < (size_t)nx * (ny - 1); ++q)
            if (d->override_y[q] >= d->n_override) throw Invalid("override index out of range");
        g.ovr_x = p.upload(d->override_x, (size_t)(nx - 1) * ny);
        g.ovr_y = p.upload(d->override_y, (size_t)nx * (ny - 1));
    }
    if (d->n_narrow > 0) {
        const int64_t nr = d->n_narrow, ne = d->narrow_ptr[nr];
        for (int64_t q = 0; q < nr; ++q) {
            if (d->narrow_pos[q] < d->off_x || d->narrow_pos[q] >= d->off_c || d->narrow_sheet[q] < 0 ||
                d->narrow_sheet[q] >= S)
                throw Invalid("narrow strip row out of range");
        }
        for (int64_t e = 0; e < ne; ++e)
            if (d->narrow_col[e] < d->off_x || d->narrow_col[e] >= d->off_c) throw Invalid("narrow strip column out of range");
        Narrow& nw = G->narrow;
        nw.nrow = nr;
        nw.pos = p.upload(d->narrow_pos, nr);
        nw.sheet = p.upload(d->narrow_sheet, nr);
        nw.rdelta = p.upload(d->narrow_rdelta, nr);
        nw.dl = p.upload(d->narrow_dl, nr);
        nw.ptr = p.upload(d->narrow_ptr, nr + 1);
        nw.col = p.upload(d->narrow_col, std::max<int64_t>(ne, 1));
        nw.val = p.upload(d->narrow_val, std::max<int64_t>(ne, 1));
        if (d->narrow_partner) {
            for (int64_t q = 0; q < nr; ++q) {
                const int64_t pp = d->narrow_partner[q];
                if (pp >= 0 && (pp < d->off_x || pp >= d->off_c || d->narrow_twin[q] < 0 ||
                                d->narrow_twin[q] >= d->n_twins))
                    throw Invalid("face partner out of range");
            }
            nw.partner = p.upload(d->narrow_partner, nr);
            nw.twin = p.upload(d->narrow_twin, nr);
            nw.tw_fac = p.upload(d->narrow_twfac, nr);
            nw.ntw = d->n_twins;
        }
        if (d->narrow_rre) {
            if (!d->narrow_twre) throw Invalid("narrow_rre needs narrow_twre");
            nw.rre = p.upload(d->narrow_rre, nr);
            nw.twre = p.upload(d->narrow_twre, nr);
        }
    }
    G->n_compact = d->n_compact;
    G->d_c2d = p.upload(d->compact_to_dense, d->n_compact);
    // the strips lead the compact order (x strips, y strips)
    G->n_strips = 0;
    while (G->n_strips < d->n_compact && d->compact_to_dense[G->n_strips] < d->off_c) ++G->n_strips;
    // FFT orientations
    const double* specs[2] = {d->spectrum_x, d->spectrum_y};
    for (int k = 0; k < 2; ++k) {
        Orient& o = G->o[k];
        o.n0 = k == 0 ? nx - 1 : nx;
        o.n1 = k == 0 ? ny : ny - 1;
        o.P0 = d->fft_p[2 * k];
        o.P1 = d->fft_p[2 * k + 1];
        if (o.P0 < 2 * o.n0 - 1 || o.P1 < 2 * o.n1 - 1) throw Invalid("FFT size below 2n - 1");
        if (o.P1 / 8 > 1024 || o.P0 / 8 > 1024) throw Invalid("FFT size too large");
        o.di = k == 0;
        o.dj = k == 1;
        o.off = k == 0 ? d->off_x : d->off_y;
        size_t q = (size_t)(o.P1 / 2 + 1) * (o.P0 / 2 + 1) * S * S;
        o.spec64 = p.upload(specs[k], q);
        std::vector<float> s32(q);
        for (size_t i = 0; i < q; ++i) s32[i] = (float)specs[k][i];
        o.spec32 = p.upload(s32.data(), q);
        for (int ax = 0; ax < 2; ++ax) {
            int P = ax == 0 ? o.P0 : o.P1;
            std::vector<c64> t64(P);
            std::vector<c32> t32(P);
            for (int m = 0; m < P; ++m) {
                double a = -2.0 * M_PI * (double)m / (double)P;
                t64[m] = mk<double>(std::cos(a), std::sin(a));
                t32[m] = mk<float>((float)t64[m].re, (float)t64[m].im);
            }
            (ax == 0 ? o.tw0_64 : o.tw1_64) = p.upload(t64.data(), P);
            (ax == 0 ? o.tw0_32 : o.tw1_32) = p.upload(t32.data(), P);
        }
        o.ld0 = (o.n0 + 15) & ~15;
        G->maxT = std::max<int64_t>(G->maxT, (int64_t)S * o.P1 * o.ld0);
    }
    // fronts
    const int nf = d->n_fronts;
    for (int f = 0; f < nf; ++f) {           // every front's panel and update matrix inside their storage
        const int64_t no = d->nown[f], nb = d->nbnd[f];
        if (no < 0 || nb < 0 || d->panel_off[f] < 0 || d->upd_off[f] < 0 ||
            d->panel_off[f] + (no + nb) * no > d->panel_total || d->upd_off[f] + nb * nb > d->upd_total)
            throw Invalid("a front's panel or update matrix lies outside panel_total / upd_total");
    }
    Fronts& F = G->F;
    F.nfront = nf;
    F.own_start = p.upload(d->own_start, nf);
    F.nown = p.upload(d->nown, nf);
    F.nbnd = p.upload(d->nbnd, nf);
    F.bnd_ptr = p.upload(d->bnd_ptr, nf + 1);
    F.bnd_idx = p.upload(d->bnd_idx, d->bnd_ptr[nf]);
    F.child_ptr = p.upload(d->child_ptr, nf + 1);
    F.child_idx = p.upload(d->child_idx, d->child_ptr[nf]);
    const int64_t nch = d->child_ptr[nf];
    F.cmap_ptr = p.upload(d->cmap_ptr, nch + 1);
    F.cmap_idx = p.upload(d->cmap_idx, d->cmap_ptr[nch]);
    F.panel_off = p.upload(d->panel_off, nf);
    F.upd_off = p.upload(d->upd_off, nf);
    F.vec_off = p.upload(d->vec_off, nf);
    F.ent_ptr = p.upload(d->ent_ptr, nf + 1);
    F.ent_row = p.upload(d->ent_row, d->ent_ptr[nf]);
    F.ent_col = p.upload(d->ent_col, d->ent_ptr[nf]);
    F.ent_s = p.upload(d->ent_s, d->ent_ptr[nf]);
    F.panel_total = d->panel_total;
    F.upd_total = d->upd_total;
    F.vec_total = d->vec_total;
    F.nsv = d->n_svalues;
    F.nfac = d->n_factor;
    F.nnode = nn;
    {
        std::vector<int64_t> ip(std::max<int64_t>(d->n_factor, 1), 0);
        for (int64_t node = 0; node < nn; ++node) {
            int64_t fi = d->perm[node];
            if (fi >= d->n_factor) throw Invalid("factor index out of range");
            if (fi >= 0) ip[fi] = node;
        }
        F.iperm = p.upload(ip.data(), ip.size());
    }
    G->level_ptr.assign(d->level_ptr, d->level_ptr + d->n_levels + 1);
    G->d_order = p.upload(d->front_order, nf);
    for (int h = 0; h < d->n_levels; ++h) {
        int mx = 1, mo = 1;
        double ent = 0;
        for (int64_t q = d->level_ptr[h]; q < d->level_ptr[h + 1]; ++q) {
            int64_t f = d->front_order[q];
            mx = std::max<int>(mx, (int)(d->nown[f] + d->nbnd[f]));
            mo = std::max<int>(mo, (int)d->nown[f]);
            ent += (double)(d->nown[f] + d->nbnd[f]) * d->nown[f];
        }
        G->level_panel.push_back(ent);
        G->level_maxnf.push_back(mx);
        G->level_maxnown.push_back(mo);
        G->max_nf = std::max(G->max_nf, mx);
    }
    {
        if (const char* e = std::getenv("GT_TILED_NF")) G->tiled_nf = std::max(1, std::atoi(e));
        std::vector<int64_t> ord;
        ord.reserve(nf);
        for (int h = 0; h < d->n_levels; ++h) {
            std::vector<int64_t> small, big;
            int bmx = 1, bmo = 1, smx = 1;
            for (int64_t q = d->level_ptr[h]; q < d->level_ptr[h + 1]; ++q) {
                const int64_t f = d->front_order[q];
                const int nff = (int)(d->nown[f] + d->nbnd[f]);
                if (nff >= G->tiled_nf) {
                    big.push_back(f);
                    bmx = std::max(bmx, nff);
                    bmo = std::max<int>(bmo, (int)d->nown[f]);
                } else {
                    small.push_back(f);
                    smx = std::max(smx, nff);
                }
            }
            ord.insert(ord.end(), small.begin(), small.end());
            ord.insert(ord.end(), big.begin(), big.end());
            G->level_nbig.push_back((int)big.size());
            G->level_bigmaxnf.push_back(bmx);
            G->level_bigmaxnown.push_back(bmo);
            G->level_smallmaxnf.push_back(smx);
        }
        G->d_forder = p.upload(ord.data(), ord.size());
        std::vector<int64_t> big;
        for (int f = 0; f < nf; ++f) {
            const int nff = (int)(d->nown[f] + d->nbnd[f]);
            if (nff < G->tiled_nf) continue;
            big.push_back(f);
            G->bigmax_nf = std::max(G->bigmax_nf, nff);
            G->bigmax_nown = std::max<int>(G->bigmax_nown, (int)d->nown[f]);
        }
        G->nbig = (int)big.size();
        G->d_bigfronts = p.upload(big.data(), big.size());
    }
    if (d->n_lowrank < 0 || d->n_lowrank > d->n_branches || d->n_lowrank > LOWRANK_MAX)
        throw Invalid("n_lowrank must be in 0 .. min(n_branches, 64)");
    G->n_lowrank = d->n_lowrank;
    G->h_branch_nodes.assign(d->branch_nodes, d->branch_nodes + 2 * d->n_branches);
    {
        // FNV-1a over everything that fixes where a factor entry lives
        uint64_t h = 1469598103934665603ull;
        auto mix = [&](const int64_t* a, int64_t len) {
            for (int64_t i = 0; i < len; ++i) {
                uint64_t v = (uint64_t)a[i];
                for (int b = 0; b < 8; ++b) {
                    h ^= (v >> (8 * b)) & 0xff;
                    h *= 1099511628211ull;
                }
            }
        };
        const int64_t sizes[5] = {d->n_factor, d->panel_total, d->upd_total, d->vec_total, (int64_t)nf};
        mix(sizes, 5);
        mix(d->perm, nn);
        mix(d->level_ptr, d->n_levels + 1);
        mix(d->front_order, nf);
        mix(d->own_start, nf);
        mix(d->nown, nf);
        mix(d->nbnd, nf);
        mix(d->bnd_ptr, nf + 1);
        mix(d->bnd_idx, d->bnd_ptr[nf]);
        mix(d->child_ptr, nf + 1);
        mix(d->child_idx, d->child_ptr[nf]);
        mix(d->panel_off, nf);
        mix(d->upd_off, nf);
        mix(d->vec_off, nf);
        G->fsig = h;
    }
    G->d_sterm_ptr = p.upload(d->sterm_ptr, d->n_svalues + 1);
    G->d_sterm_tab = p.upload(d->sterm_tab, d->sterm_ptr[d->n_svalues]);
    G->d_sterm_coef = p.upload(d->sterm_coef, d->sterm_ptr[d->n_svalues]);
    GT_CUDA(cudaDeviceSynchronize());
    GT_CUDA(cudaGetDevice(&G->device));
    *out = G.release();
    return GT_OK;
    GT_GUARD_END
}

int gt_geometry_trim(gt_geometry* G) {
    GT_GUARD_BEGIN
    if (!G) throw Invalid("null geometry");
    std::lock_guard<std::mutex> lk(G->lock);
    if (G->ws) {
        GT_CUDA(cudaDeviceSynchronize());
        G->ws.reset();
    }
    return GT_OK;
    GT_GUARD_END
}

void gt_geometry_free(gt_geometry* g) {
    if (!g) return;
    cudaDeviceSynchronize();
    delete g;
}

int gt_operators_create(gt_geometry* G, int32_t n_ops, const double* omega, const double* zs, const double* zcap,
                        const double* zbr, const double* table, gt_operators** out) {
    return gt_operators_create_shared(G, n_ops, omega, zs, zcap, zbr, table, nullptr, out);
}

int gt_operators_create_shared(gt_geometry* G, int32_t n_ops, const double* omega, const double* zs,
                               const double* zcap, const double* zbr, const double* table, const int32_t* factor_of,
                               gt_operators** out) {
    return gt_operators_create_ex(G, n_ops, omega, zs, zcap, zbr, table, factor_of, 0, out);
}

int gt_operators_create_ex(gt_geometry* G, int32_t n_ops, const double* omega, const double* zs,
                           const double* zcap, const double* zbr, const double* table, const int32_t* factor_of,
                           int32_t flags, gt_operators** out) {
    GT_GUARD_BEGIN
    if (flags & ~GT_OPS_FP32_PANELS) throw Invalid("unknown operator flags");
    if (!G || !out || n_ops < 1) throw Invalid("bad arguments");
    if (G->n_lowrank)
        throw Invalid("the geometry's last branches are a low-rank update of a base: make its operators with "
                      "gt_operators_derive");
    // No geometry lock: the factorisation reads only the geometry's fixed data (and its profiler, which has a
    // lock of its own), so a geometry's next operator set can be made while it solves with the last one.  It
    // runs on a non-blocking stream of its own, which neither the legacy default stream nor a caller's stream
    // orders it against.
    struct OwnStream {
        cudaStream_t s{};
        OwnStream() { GT_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
        ~OwnStream() { cudaStreamDestroy(s); }
    } own_stream;
    std::unique_ptr<gt_operators> O(new gt_operators());
    O->g = G;
    O->nops = n_ops;
    Pool& p = O->pool;
    const Geo& g = G->geo;
    // which operators are factorised (their own) and which factorisation each one uses
    std::vector<int> own;
    O->fslot.assign(n_ops, -1);
    for (int q = 0; q < n_ops; ++q) {
        const int src = factor_of ? factor_of[q] : q;
        if (src < 0 || src >= n_ops || (factor_of && factor_of[src] != src))
            throw Invalid("factor_of must name operators that use their own factorisation");
        if (src == q) {
            O->fslot[q] = (int)own.size();
            own.push_back(q);
        }
    }
    for (int q = 0; q < n_ops; ++q)
        if (O->fslot[q] < 0) O->fslot[q] = O->fslot[factor_of[q]];
    const int nf_ops = O->nfact = (int)own.size();
    O->own = own;
    cudaStream_t st = own_stream.s;
    O->omega = p.upload(omega, n_ops, st);
    upload_zs(O.get(), G, zs, n_ops, st);
    O->zcap = p.upload(reinterpret_cast<const c64*>(zcap), (size_t)n_ops * g.np, st);
    O->zbr = p.upload(reinterpret_cast<const c64*>(zbr), (size_t)n_ops * g.nbr, st);
    {
        // the admittance tables of the factorised operators (the preconditioner's D^-1 and the Schur values)
        std::vector<c64> t64((size_t)nf_ops * g.ntab);
        std::vector<c32> t32(t64.size());
        for (int f = 0; f < nf_ops; ++f)
            for (int e = 0; e < g.ntab; ++e) {
                const size_t src = ((size_t)own[f] * g.ntab + e) * 2, dst = (size_t)f * g.ntab + e;
                t64[dst] = mk<double>(table[src], table[src + 1]);
                t32[dst] = mk<float>((float)table[src], (float)table[src + 1]);
            }
        O->tab = p.upload(t64.data(), t64.size(), st);
        O->tab32 = p.upload(t32.data(), t32.size(), st);
        O->stiff = stiffness(t64, nf_ops, g);
        GT_CUDA(cudaStreamSynchronize(st));   // t64 and t32 go out of scope
    }
    // FP32 panels only: the FP64 factor lives in temporary memory while it is made and converted, and no FP64
    // row-major copy is made; a stiff set keeps its FP64 panels, which its FP64 preconditioner needs
    const bool keep64 = !(flags & GT_OPS_FP32_PANELS) ||
                        std::any_of(O->stiff.begin(), O->stiff.end(), [](char v) { return v != 0; });
    n_ops = nf_ops;        // the factorisation below runs over the factorised operators
    const Fronts& F = G->F;
    Pool tmp;
    c64* svals = tmp.alloc<c64>((size_t)n_ops * F.nsv);
    c64* upd = tmp.alloc<c64>((size_t)n_ops * std::max<int64_t>(F.upd_total, 1));
    int* status = tmp.alloc<int>(1);
    GT_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
    O->panel64 = (keep64 ? p : tmp).alloc<c64>((size_t)n_ops * F.panel_total);
    O->panel32 = p.alloc<c32>((size_t)n_ops * F.panel_total);
    O->panel32_rm = p.alloc<c32>((size_t)n_ops * F.panel_total);
    O->panel64_rm = keep64 ? p.alloc<c64>((size_t)n_ops * F.panel_total) : nullptr;
    O->dinv64 = p.alloc<c64>((size_t)n_ops * F.nfac);
    O->dinv32 = p.alloc<c32>((size_t)n_ops * F.nfac);
    Profiler* P = &G->prof;
    {
        Scope sc(P, "factor_assemble", st);
        launch_assemble_s(G->d_sterm_ptr, G->d_sterm_tab, G->d_sterm_coef, F.nsv, O->tab, g.ntab, svals, n_ops, st);
    }
    // every front's panel starts from zero: its own columns and its children's updates are added in (the update
    // matrices' slots are reused across levels; each front clears its own)
    GT_CUDA(cudaMemsetAsync(O->panel64, 0, (size_t)n_ops * F.panel_total * sizeof(c64), st));
    const int nlev = (int)G->level_ptr.size() - 1;
    for (int h = 0; h < nlev; ++h) {
        const int nfl = (int)(G->level_ptr[h + 1] - G->level_ptr[h]);
        const int nbig = G->level_nbig[h], nsmall = nfl - nbig;
        const int64_t* lst = G->d_forder + G->level_ptr[h];
        Scope sc(P, P->levels ? ("factor.L" + std::to_string(h)).c_str() : "factor_levels", st);
        if (nsmall) launch_factor_level(F, lst, nsmall, G->level_smallmaxnf[h], svals, O->panel64, upd, n_ops, status, st);
        if (nbig)
            launch_factor_tiled(F, lst + nsmall, nbig, G->level_bigmaxnf[h], G->level_bigmaxnown[h], svals, O->panel64,
                                upd, n_ops, status, st);
    }
    int max_nown = 1;
    for (int h = 0; h < nlev; ++h) max_nown = std::max(max_nown, G->level_maxnown[h]);
    {
        Scope sc(P, "factor_invert", st);
        launch_invert_own(F, O->panel64, max_nown, n_ops, G->tiled_nf, st);
    }
    {
        Scope sc(P, "factor_bnd_inv", st);
        launch_bnd_inv(F, O->panel64, G->max_nf, n_ops, G->tiled_nf, st);
    }
    {
        Scope sc(P, "factor_invert_tiled", st);
        launch_invert_tiled(F, G->d_bigfronts, G->nbig, G->bigmax_nf, G->bigmax_nown, O->panel64, n_ops, st);
    }
    {
        Scope sc(P, "factor_convert", st);
        launch_panel_convert(F, O->panel64, O->panel32, O->panel32_rm, O->panel64_rm, O->dinv64, O->dinv32, n_ops,
                             G->tiled_nf, st);
    }
    int h_status = 0;
    GT_CUDA(cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    P->flush(st);
    if (h_status) throw Invalid("the Schur complement has a zero or non-finite pivot (a piece of copper with no "
                                "path to its reference node?)");
    if (!keep64) O->panel64 = nullptr;   // freed with the temporary memory
    *out = O.release();
    return GT_OK;
    GT_GUARD_END
}

int gt_operators_derive(gt_geometry* G, const gt_operators* base, int32_t n_ops, const double* omega, const double* zs,
                        const double* zcap, const double* zbr, const double* table, gt_operators** out) {
    GT_GUARD_BEGIN
    if (!G || !base || !out || n_ops < 1) throw Invalid("bad arguments");
    const gt_geometry* BG = base->g;
    if (base->nlow) throw Invalid("the base is itself derived: derive from its base with all the added branches");
    const int k = G->n_lowrank;
    if (k < 1) throw Invalid("the geometry adds no branches (n_lowrank 0)");
    const Geo& g = G->geo;
    const Geo& bg = BG->geo;
    if (g.S != bg.S || g.nx != bg.nx || g.ny != bg.ny || g.np != bg.np || g.sheet != bg.sheet ||
        g.nbr != bg.nbr + k || G->fsig != BG->fsig || G->F.nfac != BG->F.nfac || G->F.nnode != BG->F.nnode)
        throw Invalid("the geometry is not the base's plus its n_lowrank last branches");
    for (int e = 0; e < 2 * bg.nbr; ++e)
        if (G->h_branch_nodes[e] != BG->h_branch_nodes[e]) throw Invalid("the base's branches must lead the geometry's");
    if (n_ops != base->nops) throw Invalid("n_ops must equal the base's operator count");
    if (!base->panel64 || !base->panel64_rm)
        throw Invalid("derive from operators that kept their FP64 panels (made without GT_OPS_FP32_PANELS)");
    if (k > G->F.nfac) throw Invalid("more added branches than kept nodes");
    std::lock_guard<std::mutex> lk(G->lock);
    std::unique_ptr<gt_operators> O(new gt_operators());
    O->g = G;
    O->nops = n_ops;
    O->nfact = base->nfact;
    O->fslot = base->fslot;
    O->own = base->own;
    O->base = base;
    Pool& p = O->pool;
    const int nf = O->nfact;
    O->omega = p.upload(omega, n_ops);
    upload_zs(O.get(), G, zs, n_ops);
    O->zcap = p.upload(reinterpret_cast<const c64*>(zcap), (size_t)n_ops * g.np);
    O->zbr = p.upload(reinterpret_cast<const c64*>(zbr), (size_t)n_ops * g.nbr);
    {
        // D^-1 of the derived stack at each factorisation's frequency (the added branches' admittances too)
        std::vector<c64> t64((size_t)nf * g.ntab);
        std::vector<c32> t32(t64.size());
        for (int f = 0; f < nf; ++f)
            for (int e = 0; e < g.ntab; ++e) {
                const size_t src = ((size_t)O->own[f] * g.ntab + e) * 2, dst = (size_t)f * g.ntab + e;
                t64[dst] = mk<double>(table[src], table[src + 1]);
                t32[dst] = mk<float>((float)table[src], (float)table[src + 1]);
            }
        O->tab = p.upload(t64.data(), t64.size());
        O->tab32 = p.upload(t32.data(), t32.size());
        O->stiff = stiffness(t64, nf, g);
    }
    O->panel64 = base->panel64;
    O->panel32 = base->panel32;
    O->panel64_rm = base->panel64_rm;
    O->panel32_rm = base->panel32_rm;
    O->dinv64 = base->dinv64;
    O->dinv32 = base->dinv32;
    O->nlow = k;
    const std::vector<int> ends(G->h_branch_nodes.begin() + 2 * bg.nbr, G->h_branch_nodes.end());
    O->low_ends = p.upload(ends.data(), ends.size());
    const int64_t nnode = G->F.nnode, ntot = (int64_t)nf * k;
    O->low_w64 = p.alloc<c64>((size_t)ntot * nnode);
    O->low_w32 = p.alloc<c32>((size_t)ntot * nnode);
    cudaStream_t st = 0;
    Profiler* P = &G->prof;
    {
        // W = S^-1 U by the base's FP64 sweeps; where the largest front is too large for the FP64 solve kernels
        // (which then serve no FP64 solve of this geometry either), by the FP32 sweeps the mixed-precision
        // solves use
        Scope sc(P, "lowrank_make", st);
        Pool tmp;
        if (solve_fits(G, sizeof(c64))) {
            lowrank_w<double>(G, base, nf, k, O->low_ends, O->low_w64, st);
            launch_lowrank_to32(O->low_w64, O->low_w32, ntot * nnode, st);
        } else {
            lowrank_w<float>(G, base, nf, k, O->low_ends, O->low_w32, st);
            launch_lowrank_to64(O->low_w32, O->low_w64, ntot * nnode, st);
        }
        // U^T W to the host; Minv = (diag(z) + U^T W)^-1 per factorisation at its frequency
        c64* gbuf = tmp.alloc<c64>((size_t)ntot * k);
        launch_lowrank_gather(O->low_w64, nnode, (int)ntot, k, O->low_ends, gbuf, st);
        std::vector<c64> hg((size_t)ntot * k);
        GT_CUDA(cudaMemcpy(hg.data(), gbuf, hg.size() * sizeof(c64), cudaMemcpyDeviceToHost));
        std::vector<c64> m64((size_t)nf * k * k);
        std::vector<c32> m32(m64.size());
        std::vector<std::complex<double>> A((size_t)k * k), X((size_t)k * k);
        for (int f = 0; f < nf; ++f) {
            const int q = O->own[f];
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) {
                    const c64 v = hg[((size_t)f * k + j) * k + i];
                    A[(size_t)i * k + j] = {v.re, v.im};
                }
            for (int i = 0; i < k; ++i) {
                const size_t zi = ((size_t)q * g.nbr + bg.nbr + i) * 2;
                A[(size_t)i * k + i] += std::complex<double>(zbr[zi], zbr[zi + 1]);
            }
            // Gauss-Jordan with partial pivoting
            for (size_t e = 0; e < X.size(); ++e) X[e] = (e / k == e % k) ? 1.0 : 0.0;
            for (int c = 0; c < k; ++c) {
                int piv = c;
                for (int r = c + 1; r < k; ++r)
                    if (std::abs(A[(size_t)r * k + c]) > std::abs(A[(size_t)piv * k + c])) piv = r;
                const std::complex<double> pv = A[(size_t)piv * k + c];
                if (!(std::abs(pv) > 0) || !std::isfinite(std::abs(pv)))
                    throw Invalid("the low-rank branch update is singular");
                if (piv != c)
                    for (int j = 0; j < k; ++j) {
                        std::swap(A[(size_t)piv * k + j], A[(size_t)c * k + j]);
                        std::swap(X[(size_t)piv * k + j], X[(size_t)c * k + j]);
                    }
                const std::complex<double> inv = 1.0 / pv;
                for (int j = 0; j < k; ++j) {
                    A[(size_t)c * k + j] *= inv;
                    X[(size_t)c * k + j] *= inv;
                }
                for (int r = 0; r < k; ++r) {
                    if (r == c) continue;
                    const std::complex<double> fct = A[(size_t)r * k + c];
                    if (fct == 0.0) continue;
                    for (int j = 0; j < k; ++j) {
                        A[(size_t)r * k + j] -= fct * A[(size_t)c * k + j];
                        X[(size_t)r * k + j] -= fct * X[(size_t)c * k + j];
                    }
                }
            }
            for (size_t e = 0; e < X.size(); ++e) {
                m64[(size_t)f * k * k + e] = mk<double>(X[e].real(), X[e].imag());
                m32[(size_t)f * k * k + e] = mk<float>((float)X[e].real(), (float)X[e].imag());
            }
        }
        O->low_m64 = p.upload(m64.data(), m64.size());
        O->low_m32 = p.upload(m32.data(), m32.size());
        GT_CUDA(cudaStreamSynchronize(st));
    }
    P->flush(st);
    *out = O.release();
    return GT_OK;
    GT_GUARD_END
}

void gt_operators_free(gt_operators* ops) {
    if (!ops) return;
    cudaDeviceSynchronize();
    delete ops;
}

int gt_to_dense(gt_geometry* G, int32_t n_cols, const double* compact, void* dense, void* stream) {
    GT_GUARD_BEGIN
    cudaStream_t st = (cudaStream_t)stream;
    Pool tmp;
    c64* d_in = tmp.upload(reinterpret_cast<const c64*>(compact), (size_t)n_cols * G->n_compact);
    GT_CUDA(cudaMemsetAsync(dense, 0, (size_t)n_cols * G->geo.n * sizeof(c64), st));
    launch_scatter(G->d_c2d, G->n_compact, d_in, G->n_compact, static_cast<c64*>(dense), G->geo.n, n_cols, st);
    GT_CUDA(cudaStreamSynchronize(st));
    return GT_OK;
    GT_GUARD_END
}

int gt_to_compact(gt_geometry* G, int32_t n_cols, const void* dense, double* compact, void* stream) {
    GT_GUARD_BEGIN
    cudaStream_t st = (cudaStream_t)stream;
    Pool tmp;
    c64* d_out = tmp.alloc<c64>((size_t)n_cols * G->n_compact);
    launch_gather(G->d_c2d, G->n_compact, static_cast<const c64*>(dense), G->geo.n, d_out, G->n_compact, n_cols, st);
    GT_CUDA(cudaMemcpyAsync(compact, d_out, (size_t)n_cols * G->n_compact * sizeof(c64), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    return GT_OK;
    GT_GUARD_END
}

int gt_solve_device(gt_geometry* G, gt_operators* ops, int32_t n_cols, const int32_t* col_op, const void* rhs_device,
                    const gt_solve_opts* opts, void* x_device, int32_t* its_out, double* resid_out, void* stream) {
    GT_GUARD_BEGIN
    if (!G || !ops || !opts || n_cols < 1) throw Invalid("bad arguments");
    std::lock_guard<std::mutex> lk(G->lock);
    cudaStream_t st = (cudaStream_t)stream;
    gt_solve_opts eo = *opts;
    eo.precision = effective_precision(G, ops, n_cols, col_op, eo.precision);
    opts = &eo;
    ensure_ws(G, n_cols, opts->restart, opts->precision, std::max(1, opts->outer_k), st);
    Workspace& W = *G->ws;
    GT_CUDA(cudaMemcpyAsync(W.b64, rhs_device, (size_t)n_cols * G->geo.n * sizeof(c64), cudaMemcpyDeviceToDevice, st));
    if (opts->use_guess)
        GT_CUDA(cudaMemcpyAsync(W.x64, x_device, (size_t)n_cols * G->geo.n * sizeof(c64), cudaMemcpyDeviceToDevice, st));
    int rc = run_solve(G, ops, n_cols, col_op, opts, its_out, resid_out, st);
    GT_CUDA(cudaMemcpyAsync(x_device, W.x64, (size_t)n_cols * G->geo.n * sizeof(c64), cudaMemcpyDeviceToDevice, st));
    GT_CUDA(cudaStreamSynchronize(st));
    check_device_waits();
    if (rc != GT_OK) gt::set_error("GMRES did not converge for at least one column");
    return rc;
    GT_GUARD_END
}

int gt_solve(gt_geometry* G, gt_operators* ops, int32_t n_cols, const int32_t* col_op, const double* rhs,
             const gt_solve_opts* opts, double* x_out, int32_t* its_out, double* resid_out, void* stream) {
    GT_GUARD_BEGIN
    if (!G || !ops || !opts || n_cols < 1 || !rhs || !x_out) throw Invalid("bad arguments");
    std::lock_guard<std::mutex> lk(G->lock);
    cudaStream_t st = (cudaStream_t)stream;
    gt_solve_opts eo = *opts;
    eo.precision = effective_precision(G, ops, n_cols, col_op, eo.precision);
    opts = &eo;
    ensure_ws(G, n_cols, opts->restart, opts->precision, std::max(1, opts->outer_k), st);
    Workspace& W = *G->ws;
    const int64_t nc = G->n_compact;
    Pool tmp;
    c64* d_c = tmp.alloc<c64>((size_t)n_cols * nc);
    GT_CUDA(cudaMemcpyAsync(d_c, rhs, (size_t)n_cols * nc * sizeof(c64), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaMemsetAsync(W.b64, 0, (size_t)n_cols * G->geo.n * sizeof(c64), st));
    launch_scatter(G->d_c2d, nc, d_c, nc, W.b64, G->geo.n, n_cols, st);
    if (opts->use_guess) {
        GT_CUDA(cudaMemcpyAsync(d_c, x_out, (size_t)n_cols * nc * sizeof(c64), cudaMemcpyHostToDevice, st));
        GT_CUDA(cudaMemsetAsync(W.x64, 0, (size_t)n_cols * G->geo.n * sizeof(c64), st));
        launch_scatter(G->d_c2d, nc, d_c, nc, W.x64, G->geo.n, n_cols, st);
    }
    int rc = run_solve(G, ops, n_cols, col_op, opts, its_out, resid_out, st);
    launch_gather(G->d_c2d, nc, W.x64, G->geo.n, d_c, nc, n_cols, st);
    GT_CUDA(cudaMemcpyAsync(x_out, d_c, (size_t)n_cols * nc * sizeof(c64), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    check_device_waits();
    if (rc != GT_OK) gt::set_error("GMRES did not converge for at least one column");
    return rc;
    GT_GUARD_END
}

int gt_memory(gt_geometry* G, int32_t n_cols, const gt_solve_opts* opts, int64_t* need, int64_t* held,
              int64_t* free_bytes, int64_t* total_bytes) {
    GT_GUARD_BEGIN
    if (!G || !opts || n_cols < 1) throw Invalid("bad arguments");
    if (opts->restart < 1 || opts->restart > 250) throw Invalid("restart must be in 1..250");
    std::lock_guard<std::mutex> lk(G->lock);
    // the workspace plus gt_solve's compact staging of the right-hand sides and solutions
    const size_t ws = ws_bytes(G, n_cols, opts->restart, opts->precision, std::max(1, opts->outer_k));
    if (need) *need = (int64_t)(ws + (size_t)n_cols * G->n_compact * sizeof(c64));
    if (held) *held = G->ws ? (int64_t)G->ws->pool.bytes : 0;
    size_t fr = 0, tot = 0;
    if (free_bytes || total_bytes) GT_CUDA(cudaMemGetInfo(&fr, &tot));
    if (free_bytes) *free_bytes = (int64_t)fr;
    if (total_bytes) *total_bytes = (int64_t)tot;
    return GT_OK;
    GT_GUARD_END
}

int gt_apply(gt_geometry* G, gt_operators* ops, int32_t kind, int32_t precision, int32_t n_cols, const int32_t* col_op,
             const double* x, double* y, void* stream) {
    GT_GUARD_BEGIN
    if (!G || !ops || n_cols < 1 || kind < 0 || kind > 2) throw Invalid("bad arguments");
    std::lock_guard<std::mutex> lk(G->lock);
    for (int c = 0; c < n_cols; ++c)
        if (col_op[c] < 0 || col_op[c] >= ops->nops) throw Invalid("column operator index out of range");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = G->geo.n, nc = G->n_compact;
    Pool tmp;
    c64* d_c = tmp.upload(reinterpret_cast<const c64*>(x), (size_t)n_cols * nc);
    c64* xin = tmp.alloc<c64>((size_t)n_cols * n);
    c64* yout = tmp.alloc<c64>((size_t)n_cols * n);
    int* d_op = tmp.upload(col_op, n_cols);
    GT_CUDA(cudaMemsetAsync(xin, 0, (size_t)n_cols * n * sizeof(c64), st));
    GT_CUDA(cudaMemsetAsync(yout, 0, (size_t)n_cols * n * sizeof(c64), st));
    launch_scatter(G->d_c2d, nc, d_c, nc, xin, n, n_cols, st);
    std::vector<int> h_op(col_op, col_op + n_cols), h_pc(n_cols);
    for (int c = 0; c < n_cols; ++c) h_pc[c] = ops->fslot[h_op[c]];
    int* d_pc = tmp.upload(h_pc.data(), n_cols);
    // kind 1 groups columns by factorisation: require them sorted
    for (int c = 1; c < n_cols; ++c)
        if (kind == 1 && h_pc[c] < h_pc[c - 1]) throw Invalid("preconditioner columns must be sorted by operator");
    auto run = [&](auto tag) {
        using R = decltype(tag);
        cx<R>* xi;
        cx<R>* yo;
        if constexpr (sizeof(R) == 8) {
            xi = xin;
            yo = yout;
        } else {
            xi = tmp.alloc<c32>((size_t)n_cols * n);
            yo = tmp.alloc<c32>((size_t)n_cols * n);
            // round the input to FP32 through a refine-style copy: y = 1.0 * x
            std::vector<c64> hx((size_t)n_cols * n);
            GT_CUDA(cudaStreamSynchronize(st));          // xin was made on the caller's stream
            GT_CUDA(cudaMemcpy(hx.data(), xin, hx.size() * sizeof(c64), cudaMemcpyDeviceToHost));
            std::vector<c32> h32(hx.size());
            for (size_t i = 0; i < hx.size(); ++i) h32[i] = cvt<float>(hx[i]);
            GT_CUDA(cudaMemcpy(xi, h32.data(), h32.size() * sizeof(c32), cudaMemcpyHostToDevice));
        }
        if (kind == 0 || kind == 2) {
            cx<R>* T = tmp.alloc<cx<R>>((size_t)n_cols * G->maxT);
            matvec<R>(G, ops, xi, nullptr, yo, n, n_cols, d_op, kind == 0 ? 0 : 2, T, st);
        } else {
            std::vector<int> gptr, gslot, gop, all(n_cols);
            for (int c = 0; c < n_cols; ++c) all[c] = c;
            const int gmax = group_max(G, sizeof(cx<R>));
            make_groups(all, h_pc, gmax, gptr, gslot, gop);
            int* g0 = tmp.upload(gptr.data(), gptr.size());
            int* g1 = tmp.upload(gslot.data(), gslot.size());
            int* g2 = tmp.upload(gop.data(), gop.size());
            Groups grp{(int)gop.size(), g0, g1, g2};
            cx<R>* zf = tmp.alloc<cx<R>>((size_t)n_cols * G->F.nfac);
            cx<R>* yf = tmp.alloc<cx<R>>((size_t)n_cols * G->F.nfac);
            cx<R>* uv = tmp.alloc<cx<R>>((size_t)n_cols * std::max<int64_t>(G->F.vec_total, 1));
            cx<R>* sdv = tmp.alloc<cx<R>>((size_t)n_cols * G->F.nnode);
            GT_CUDA(cudaMemsetAsync(sdv, 0, (size_t)n_cols * G->F.nnode * sizeof(cx<R>), st));
            precond<R>(G, ops, xi, n, yo, n, n_cols, d_pc, grp, gmax, zf, yf, uv, sdv, st);
        }
        if constexpr (sizeof(R) == 4) {
            std::vector<c32> h32((size_t)n_cols * n);
            GT_CUDA(cudaStreamSynchronize(st));
            GT_CUDA(cudaMemcpy(h32.data(), yo, h32.size() * sizeof(c32), cudaMemcpyDeviceToHost));
            std::vector<c64> h64(h32.size());
            for (size_t i = 0; i < h32.size(); ++i) h64[i] = cvt<double>(h32[i]);
            GT_CUDA(cudaMemcpy(yout, h64.data(), h64.size() * sizeof(c64), cudaMemcpyHostToDevice));
        }
    };
    if (precision == 1) run(double{});
    else run(float{});
    launch_gather(G->d_c2d, nc, yout, n, d_c, nc, n_cols, st);
    GT_CUDA(cudaMemcpyAsync(y, d_c, (size_t)n_cols * nc * sizeof(c64), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    check_device_waits();
    return GT_OK;
    GT_GUARD_END
}

int gt_strip_coupling(gt_geometry* G, const double* sheet_z, const double* sheet_t, double pitch, int32_t n_seg,
                      const double* segments, double* psi, int64_t* n_strips) {
    GT_GUARD_BEGIN
    if (!G || !sheet_z || !sheet_t || !psi || n_seg < 0 || (n_seg > 0 && !segments) || !(pitch > 0))
        throw Invalid("bad arguments");
    std::lock_guard<std::mutex> lk(G->lock);
    const int64_t ns = G->n_strips;
    if (n_strips) *n_strips = ns;
    Pool tmp;
    const int S = G->geo.S;
    double* dz = tmp.upload(sheet_z, S);
    double* dt = tmp.upload(sheet_t, S);
    double* dseg = n_seg ? tmp.upload(segments, (size_t)n_seg * 8) : nullptr;
    double* dpsi = tmp.alloc<double>(std::max<int64_t>(ns, 1));
    cudaStream_t st = 0;
    if (n_seg == 0) GT_CUDA(cudaMemsetAsync(dpsi, 0, std::max<int64_t>(ns, 1) * sizeof(double), st));
    else launch_strip_coupling(G->geo, G->d_c2d, ns, dz, dt, pitch, dseg, n_seg, dpsi, st);
    GT_CUDA(cudaMemcpy(psi, dpsi, ns * sizeof(double), cudaMemcpyDeviceToHost));
    return GT_OK;
    GT_GUARD_END
}

int gt_node_field(gt_geometry* G, int32_t n_cols, const void* x_device, double pitch, void* kx_device,
                  void* ky_device, void* stream) {
    GT_GUARD_BEGIN
    if (!G || n_cols < 1 || !x_device || !kx_device || !ky_device || !(pitch > 0)) throw Invalid("bad arguments");
    if (G->geo.NL != G->geo.S) throw Invalid("node fields of face sheets are summed per layer on the host");
    std::lock_guard<std::mutex> lk(G->lock);
    cudaStream_t st = (cudaStream_t)stream;
    launch_node_field(G->geo, static_cast<const c64*>(x_device), G->geo.n, n_cols, pitch, static_cast<c64*>(kx_device),
                      static_cast<c64*>(ky_device), st);
    GT_CUDA(cudaStreamSynchronize(st));
    return GT_OK;
    GT_GUARD_END
}

int gt_moment(gt_geometry* G, int32_t n_cols, const void* x_device, const double* sheet_z, double pitch, double* m,
              void* stream) {
    GT_GUARD_BEGIN
    if (!G || n_cols < 1 || !x_device || !sheet_z || !m || !(pitch > 0)) throw Invalid("bad arguments");
    if (G->geo.NL != G->geo.S) throw Invalid("the moment of face sheets is taken on the host");
    std::lock_guard<std::mutex> lk(G->lock);
    cudaStream_t st = (cudaStream_t)stream;
    Pool tmp;
    double* dz = tmp.upload(sheet_z, G->geo.S);
    c64* dm = tmp.alloc<c64>((size_t)n_cols * 3);
    launch_moment(G->geo, static_cast<const c64*>(x_device), G->geo.n, n_cols, dz, pitch, dm, st);
    GT_CUDA(cudaStreamSynchronize(st));
    GT_CUDA(cudaMemcpy(m, dm, (size_t)n_cols * 3 * sizeof(c64), cudaMemcpyDeviceToHost));
    return GT_OK;
    GT_GUARD_END
}

int gt_kernel_spectrum(int32_t n_axial, int32_t n_lateral, double d, double dz, int32_t P0, int32_t P1,
                       const double* near, int32_t n_near, double* quad) {
    GT_GUARD_BEGIN
    if (n_axial < 1 || n_lateral < 1 || !(d > 0) || !(dz >= 0) || !near || n_near < 1 || !quad)
        throw Invalid("bad arguments");
    if (!good_fft_size(P0) || !good_fft_size(P1) || P0 < 2 * n_axial - 1 || P1 < 2 * n_lateral - 1)
        throw Invalid("FFT sizes must be 2^a or 3*2^a (a >= 3) and cover 2n - 1");
    kernel_spectrum(n_axial, n_lateral, d, dz, P0, P1, near, n_near, quad);
    return GT_OK;
    GT_GUARD_END
}

int gt_profile(gt_geometry* G, char* names, int32_t names_cap, double* ms, double* bytes, int32_t* launches,
               int32_t cap) {
    if (!G) return 0;
    std::lock_guard<std::mutex> lk(G->prof.lock);
    if (names == nullptr && cap < 0) {  // toggle: cap = -1 off, -2 on (and reset), -3 on with levels
        G->prof.on = cap <= -2;
        G->prof.levels = cap == -3;
        G->prof.acc.clear();
        return 0;
    }
    std::string s;
    int k = 0;
    for (auto& kv : G->prof.acc) {
        if (k >= cap) break;
        if (!s.empty()) s += ",";
        s += G->prof.names[kv.first];
        ms[k] = kv.second.ms;
        bytes[k] = kv.second.bytes;
        launches[k] = kv.second.launches;
        ++k;
    }
    if (names && names_cap > 0) {
        std::strncpy(names, s.c_str(), names_cap - 1);
        names[names_cap - 1] = 0;
    }
    return k;
}

}  // extern "C"
