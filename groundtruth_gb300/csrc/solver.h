// Per-slot GMRES state shared by gmres.cu and the driver.
#pragma once
#include "kernels.h"

namespace gt {

struct GmresState {
    int nslot, m, ldh, max_its;
    double reorth_ratio;
    c64* H;            // [slot][m][m+1] rotated Hessenberg columns
    double* cs;        // [slot][m]
    c64* sn;           // [slot][m]
    c64* g;            // [slot][m+1]
    c64* hvec;         // [slot][ldh] first-pass projections, |w|^2 at index j+1
    c64* h2vec;        // [slot][ldh] second-pass projections
    c64* y;            // [slot][ldh] least-squares solution
    c64* hn2;          // [slot] |w|^2 after the first pass
    c64* hn2b;         // [slot] after the second
    int* it;           // [slot] iterations of the current cycle
    int* its_total;    // [slot] iterations of the column so far (copied in and out per cycle)
    int* active;       // [slot]
    int* reorth;       // [slot]
    double* eta;       // [slot] the cycle's relative target
    double* inv_hn;    // [slot]
    double* resid_est; // [slot]
};

template <typename R, typename B = cx<R>> struct GmresStateT {
    int nslot;
    int* active;
    double* inv_hn;
    B* V;              // [slot][m+1][ldv], times scale
    cx<R>* w;          // [slot][ldv]
    int64_t ldv, lds;
    R scale;           // the basis scale (1 unless B is a narrower type than cx<R>)
    cx<R>* vcur;       // [slot][ldv]: the newest basis vector as stored, unscaled (B != cx<R> only)
};

void launch_dgks(const GmresState& s, int j, cudaStream_t st);
void launch_givens(const GmresState& s, int j, cudaStream_t st);
template <typename R, typename B> void launch_scale(const GmresStateT<R, B>& s, int j, int64_t n, cudaStream_t st);
void launch_hsolve(const GmresState& s, cudaStream_t st);
template <typename R, typename B>
void launch_init_cycle(const GmresStateT<R, B>& s, const c64* r, int64_t ldr, const int* slot_col, const double* rho,
                       int64_t n, cudaStream_t st);
void launch_init_state(const GmresState& s, const int* slot_col, const double* rho, const double* bnorm, double tol,
                       double inner_tol, cudaStream_t st);
template <typename R>
void launch_refine(c64* x, int64_t ldx, const cx<R>* e, int64_t lde, const int* slot_col, const double* rho, int64_t n,
                   int nslot, cudaStream_t st);
void launch_any_active(const int* active, int n, int* flag, cudaStream_t st);
// dst[slot_col[s]] = src[s] (precision R -> FP64), s < nslot
template <typename R>
void launch_to64(c64* dst, int64_t ldd, const cx<R>* src, int64_t lds, const int* slot_col, int64_t n, int nslot,
                 cudaStream_t st);
// the GCR direction of each active column scaled to a unit product: p /= |q|, q /= |q| (|q|^2 in nu2)
void launch_gcr_scale(c64* p, c64* q, int64_t ld, const c64* nu2, const int* active, int64_t n, int ncol,
                      cudaStream_t st);
void launch_sqrt_norms(const c64* nrm2, int ld, int n, double* out, cudaStream_t st);
// out[i] = sqrt(nrm2[i * ld].re) for active i only
void launch_sqrt_norms_active(const c64* nrm2, int ld, int n, const int* active, double* out, cudaStream_t st);

}  // namespace gt
