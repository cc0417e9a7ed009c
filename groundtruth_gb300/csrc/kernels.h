// Launch interfaces between the kernel files and the host driver (api.cu).
#pragma once
#include "common.cuh"

namespace gt {

// The geometry as the kernels see it (device pointers, sizes).
struct Geo {
    int S, nx, ny, np, nbr, sheet;
    int NL;                      // node layers (S minus the split layers' lower-face sheets)
    const int* sheet_layer;      // [S] the layer whose nodes each sheet's strips join
    int64_t n, off_x, off_y, off_c, off_b, off_v;
    const uint8_t* mask;
    const uint8_t* code_x;
    const uint8_t* code_y;
    const int* pair_layers;      // [np*2]
    const int* branch_nodes;     // [nbr*2] dense node index
    const int* node_br_ptr;      // [S*nx*ny + 1] CSR of branch ends per dense node
    const int* node_br_idx;      // branch index + 1, negated for the b end
    const int64_t* perm;         // dense node -> factor index or -1
    int64_t nfac;
    int ntab, tab_cap0, tab_br0;
    // positions whose strips are not all full width (their own S x S blocks of D^-1 at tab_ovr0 + idx S S):
    // per x / y strip position the block index or -1 (null: none)
    const int* ovr_x;
    const int* ovr_y;
    int tab_ovr0;
    // per capacitance cell [np][nx][ny] the share of the cell's area both planes' copper covers (a cell of
    // admittance share / z_cap); null: every cell whole
    const double* cap_fill;
};

// The narrow strips' corrections to the system product (narrow.cu): rows at dense positions pos[q] of sheet
// sheet[q], resistance factor rdelta = 1/width - 1, self-inductance change dl (H), and the mutual changes
// M[q, col[e]] = val[e] (H) for e in ptr[q] .. ptr[q+1]
struct Narrow {
    int64_t nrow = 0;
    const int64_t* pos = nullptr;
    const int* sheet = nullptr;
    const double* rdelta = nullptr;
    const double* dl = nullptr;
    const int64_t* ptr = nullptr;
    const int64_t* col = nullptr;
    const double* val = nullptr;
    // a split layer's face strips: the partner face's strip (dense position, -1: none), the split layer's index
    // into the per-operator face couplings and the factor 1 / width: out[p] += z_mut fac x[partner]
    const int64_t* partner = nullptr;
    const int* twin = nullptr;
    const double* tw_fac = nullptr;
    int ntw = 0;
    // resistance factors (null: none): out[p] += rre Re(z) x[p] + twre Re(z_mut) x[partner]
    const double* rre = nullptr;
    const double* twre = nullptr;
};
template <typename R>
void launch_narrow(const Narrow& nw, const cx<R>* x, cx<R>* out, int64_t ld, int ncol, int S, const int* col_op,
                   const double* omega, const c64* zs, const c64* zmut, int mode, const int* col_list,
                   cudaStream_t st);

template <typename R> struct LpArgs {
    const cx<R>* x;
    const cx<R>* rhs;
    cx<R>* out;
    int64_t ld, off, off_v;
    int S, n0, n1, nx, ny, di, dj, P0, P1, ncol;
    const cx<R>* tw0;      // twiddles of the column length P0
    const cx<R>* tw1;      // of the row length P1
    const R* spec;         // (Q1, Q0, S, S)
    cx<R>* T;              // [ncol][S][P1][ldt]
    int ldt;               // T's row stride (>= n0; a multiple of 16 so the row passes move aligned 128-byte runs)
    const uint8_t* mask;
    const int* col_op;
    const double* omega;
    const c64* zs;
    int mode;
    const int* col_list;
    const int* sheet_layer;   // [S] node layer of each sheet's strips (null: the sheet itself)
    int rows;              // rows per block of the row passes (0: default)
    int bt;                // columns per block of the column pass (0: default)
};

template <typename R> void launch_lp(const LpArgs<R>& a, cudaStream_t st);
// TMA waits of the L_p pass that gave up since the last call (and clears the count); read once the kernels are done
unsigned int lp_take_wait_timeouts();
// one of the three passes (0: row FFTs, 1: column FFTs + spectrum, 2: inverse row FFTs + epilogue)
template <typename R> void launch_lp_pass(const LpArgs<R>& a, int pass, cudaStream_t st);
// the launch shapes launch_lp would use for these arguments
template <typename R> void lp_shapes(const LpArgs<R>& a, int* rows, int* bt);

// capacitance / branch / node rows of the system product (mode 0: K x, 1: rhs - K x); also zeroes the
// padding between segments
template <typename R>
void launch_tail(const Geo& g, const cx<R>* x, const cx<R>* rhs, cx<R>* out, int64_t ld, int ncol, const int* col_op,
                 const c64* zcap, const c64* zbr, int mode, const int* col_list, cudaStream_t st);

// preconditioner: s = r_V - Ar^T D^-1 r_1 into factor order (sd [col][nfac]); then, with y in node order in
// sd [col][S*nx*ny] (zero at nodes that are not kept), out = [D^-1 (r_1 + Ar y); y]
template <typename R>
void launch_pc_node(const Geo& g, const cx<R>* r, int64_t ld, cx<R>* sd, int ncol, const int* col_op,
                    const cx<R>* tab, const int* col_list, cudaStream_t st);
template <typename R>
void launch_pc_strip(const Geo& g, const cx<R>* r, int64_t ldr, const cx<R>* sd, cx<R>* out, int64_t ldo, int ncol,
                     const int* col_op, const cx<R>* tab, const int* col_list, cudaStream_t st);

// psi of the first ns compact entries (the strips): segments [nseg][8] (a, b, width, current), device FP64
void launch_strip_coupling(const Geo& g, const int64_t* c2d, int64_t ns, const double* sheet_z, const double* sheet_t,
                           double d, const double* segs, int nseg, double* psi, cudaStream_t st);

// post-solve outputs from dense FP64 solutions [col][ld]: node fields kx / ky [col][S][nx][ny]; moments [col][3]
void launch_node_field(const Geo& g, const c64* x, int64_t ld, int ncol, double d, c64* kx, c64* ky, cudaStream_t st);
void launch_moment(const Geo& g, const c64* x, int64_t ld, int ncol, const double* zs, double d, c64* m,
                   cudaStream_t st);

// the real (P0/2+1) x (P1/2+1) spectrum quadrant of a strip kernel (host in / out, device work)
void kernel_spectrum(int na, int nl, double d, double dz, int P0, int P1, const double* near_h, int nnear,
                     double* quad_h);

// compact <-> dense
void launch_scatter(const int64_t* c2d, int64_t ncomp, const c64* in, int64_t ldin, c64* out, int64_t ldout, int ncol,
                    cudaStream_t st);
void launch_gather(const int64_t* c2d, int64_t ncomp, const c64* in, int64_t ldin, c64* out, int64_t ldout, int ncol,
                   cudaStream_t st);

// --- multifrontal factorisation and solves
struct Fronts {
    int nfront;
    const int64_t* own_start;
    const int64_t* nown;
    const int64_t* nbnd;
    const int64_t* bnd_ptr;
    const int64_t* bnd_idx;
    const int64_t* child_ptr;
    const int64_t* child_idx;
    const int64_t* cmap_ptr;
    const int64_t* cmap_idx;
    const int64_t* panel_off;
    const int64_t* upd_off;
    const int64_t* vec_off;
    const int64_t* ent_ptr;
    const int* ent_row;
    const int* ent_col;
    const int64_t* ent_s;
    int64_t panel_total, upd_total, vec_total, nsv, nfac;
    const int64_t* iperm;        // factor index -> dense node index
    int64_t nnode;               // dense nodes S * nx * ny (the node-ordered vectors' length)
};

void launch_assemble_s(const int64_t* ptr, const int* tab_idx, const double* coef, int64_t nsv, const c64* table,
                       int ntab, c64* svals, int nops, cudaStream_t st);
// one elimination level: fronts front_list[0..nf) for each operator
void launch_factor_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, const c64* svals,
                         c64* panel, c64* upd, int nops, int* status, cudaStream_t st);
// one level's large fronts (blocked elimination over many CTAs); the fronts start zeroed
void launch_factor_tiled(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                         const c64* svals, c64* panel, c64* upd, int nops, int* status, cudaStream_t st);
// each front's own block replaced by its inverse (in place, FP64; the unit diagonal and the pivots untouched)
void launch_invert_own(const Fronts& F, c64* panel, int max_nown, int nops, int tiled_nf, cudaStream_t st);
// each front's boundary rows replaced by -L_bnd Linv_own (in place, FP64; after launch_invert_own)
void launch_bnd_inv(const Fronts& F, c64* panel, int max_nbnd, int nops, int tiled_nf, cudaStream_t st);
// both at once for the listed (large) fronts, blocked over many CTAs; the two above skip fronts of tiled_nf rows
// or more, and panel_convert takes their inverse in place
void launch_invert_tiled(const Fronts& F, const int64_t* front_list, int nfront, int max_nf, int max_nown, c64* panel,
                         int nops, cudaStream_t st);
// the solve panels: own blocks get a unit diagonal and zeros above it (pivot reciprocals to d64 / d32,
// [op][nfac]); FP32 column-major, FP32 and FP64 row-major copies
void launch_panel_convert(const Fronts& F, c64* p64, c32* p32, c32* r32, c64* r64, c64* d64, c32* d32, int nops, int tiled_nf,
                          cudaStream_t st);

// triangular solves, per level; groups of columns sharing an operator
struct Groups {
    int ngroup;
    const int* gptr;       // group g: columns gslot[gptr[g] .. gptr[g+1])
    const int* gslot;
    const int* op;
};
// forward: own rows from s in factor order (sf), results to z (factor order) and the update vectors (wasm:
// factor-ordered scratch for fronts assembled ahead of a split product, may be sf itself);
// backward: reads z and the ancestors' y, writes y (factor order) and sd (node order)
template <typename R>
void launch_fwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                      const cx<R>* panel, const cx<R>* dinv, const cx<R>* sf, cx<R>* z, cx<R>* uvec, cx<R>* wasm,
                      const Groups& G, int gmax, cudaStream_t st);
template <typename R>
void launch_bwd_level(const Fronts& F, const int64_t* front_list, int nf_level, int max_nf, int max_nown,
                      const cx<R>* panel_rm, const cx<R>* z, cx<R>* y, cx<R>* sd, const Groups& G, int gmax,
                      cudaStream_t st);

// --- low-rank branch update of a factorised Schur complement (woodbury.cu)
constexpr int LOWRANK_MAX = 64;      // branches one derived operator set may add
// y (node order, sd [col][nnode]) -= W Minv (U^T y) per column: W [fact][k][nnode], Minv [fact][k][k],
// col_fact[col] the factorisation; cbuf [col][ldc] scratch for the k coefficients
template <typename R>
void launch_lowrank(cx<R>* sd, int64_t nnode, int ncol, int k, const int* ends, const cx<R>* w, const cx<R>* minv,
                    const int* col_fact, const int* col_list, cx<R>* cbuf, int64_t ldc, cudaStream_t st);
// U e_j in factor order for the columns c0 .. c0+ncol of (factorisation, branch) pairs (j = c mod k)
template <typename R>
void launch_lowrank_rhs(cx<R>* s, int64_t nfac, int c0, int ncol, int k, const int* ends, const int64_t* perm,
                        cudaStream_t st);
// U^T W entries g[c][i] of ncol node-ordered columns
void launch_lowrank_gather(const c64* w, int64_t nnode, int ncol, int k, const int* ends, c64* g, cudaStream_t st);
void launch_lowrank_to32(const c64* a, c32* b, int64_t n, cudaStream_t st);
// dst[c] = src[c] (n entries, converted) for c = list[0 .. nslot) (0 .. nslot when list is null)
template <typename D, typename S>
void launch_recast(cx<D>* dst, int64_t ldd, const cx<S>* src, int64_t lds, const int* list, int64_t n, int nslot,
                   cudaStream_t st);
void launch_lowrank_to64(const c32* a, c64* b, int64_t n, cudaStream_t st);

// --- Krylov vector work (batched, one basis per slot)
// A basis entry stored in FP16 (real and imaginary halves), scaled by the basis scale so that the entries
// of a unit vector of length n sit near 1, inside FP16's normal range.
struct h16c {
    __half2 v;
};
// Basis vectors are stored as B (cx<R>, or h16c for R = float) times the scale; vs = 1 / scale undoes it.
template <typename R, typename B>
void launch_dots(const B* V, int64_t ldv, int64_t lds, int nv, const cx<R>* w, int64_t ldw, int64_t n, int nslot,
                 const int* active, c64* partial, int nchunk, cudaStream_t st, R vs = R(1));
void launch_reduce(const c64* partial, int nchunk, int nv, int nslot, const int* active, c64* out, int ldo, int mode,
                   cudaStream_t st);
// partial (if not null): |w|^2 per update chunk, update_chunks(n) per slot
int update_chunks(int64_t n);
template <typename R, typename B>
void launch_update(const B* V, int64_t ldv, int64_t lds, int nv, const c64* h, int ldh, cx<R>* w, int64_t ldw,
                   int64_t n, int nslot, const int* active, c64* partial, int sign, cudaStream_t st, R vs = R(1));

}  // namespace gt
