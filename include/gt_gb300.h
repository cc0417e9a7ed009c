/*
 * gt_gb300.h - C ABI of the GB300 (sm_103a) PEEC plane-current solver.
 *
 * The library replaces the per-net, per-frequency solve of GroundTruth's quasi-static PEEC solver:
 *   PlaneStack.__init__ / _topology / _kernels   src/groundtruth/solver/peec.py:1559-1593, 1596-1656, 1941-1988
 *   PlaneStack.operator / _factorise             src/groundtruth/solver/peec.py:2227-2290, 2345-2445
 *   PlaneStack.solve / _solve / _gmres           src/groundtruth/solver/peec.py:2513-2607, 3093-3224
 *   _HostMath.matvec / precond                   src/groundtruth/solver/peec.py:3043-3083
 *   gpu.TorchMath (the reference's device seam)  src/groundtruth/solver/gpu.py:471-573
 *
 * The reference is pure Python and has no FFI of its own; these entry points are what its backend seam
 * (_solve_here choosing a math object, peec.py:2544-2558) would bind through ctypes: geometry handles built
 * once per PlaneStack, operator handles once per factorised frequency, and batched solves.  All arguments
 * are plain pointers and sizes.  Complex arrays are interleaved (re, im) doubles.  Host pointers unless a
 * name says _device.  Every entry returns a gt_status; gt_last_error() describes the last failure of the
 * calling thread.  No entry point falls back to the CPU.
 */
#ifndef GT_GB300_H
#define GT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gt_status {
    GT_OK = 0,
    GT_NOT_CONVERGED = 1,     /* peec.SolverError "GMRES did not converge" (peec.py:2599-2600) */
    GT_OUT_OF_MEMORY = 2,     /* MemoryError: the relief ladder's signal (peec.py:2425-2430) */
    GT_TIMEOUT = 3,           /* a bounded device wait ran out */
    GT_INVALID_ARGUMENT = 4,  /* malformed sizes or indices (ValueError / SolverError at the caller) */
    GT_DEVICE_ERROR = 5       /* any other CUDA failure */
} gt_status;

typedef struct gt_geometry gt_geometry;
typedef struct gt_operators gt_operators;

/* Everything of a PlaneStack that does not depend on the frequency, in the device's dense on-grid layout:
 * an unknown vector is [X (S,nx-1,ny) | Y (S,nx,ny-1) | C (n_pairs,nx,ny) | B (n_branches) | V (S,nx,ny)],
 * each segment at its offset, masked entries zero.  Replaces PlaneStack.__init__ (peec.py:1559-1593). */
typedef struct gt_geometry_desc {
    int32_t n_sheets, nx, ny, n_pairs, n_branches;
    int32_t precond_sheet;              /* 0: diagonal D (precond "diag"), 1: per-position blocks ("sheet") */
    int64_t n_dense;                    /* dense vector length */
    int64_t off_x, off_y, off_c, off_b, off_v;
    const uint8_t* mask;                /* [n_dense] 1 where an unknown lives (strips, caps, branches, kept nodes) */
    const uint8_t* code_x;              /* [(nx-1)*ny] bit k: sheet k has an x strip at the position */
    const uint8_t* code_y;              /* [nx*(ny-1)] */
    const int32_t* pair_layers;         /* [n_pairs*2] upper, lower sheet */
    const int32_t* branch_nodes;        /* [n_branches*2] dense node index (k*nx*ny + i*ny + j) of ends a, b */
    int64_t n_compact;                  /* nb + n_keep: the reference's unknown count (peec.py:2565) */
    const int64_t* compact_to_dense;    /* [n_compact] */
    int32_t fft_p[4];                   /* x: P0, P1; y: P0, P1 (each 2^a or 3*2^a, a >= 3) */
    const double* spectrum_x;           /* [(P1/2+1)*(P0/2+1)*S*S] real kernel quadrant, scaled 1/(P0*P1) */
    const double* spectrum_y;
    /* Schur complement S = Ar^T D^-1 Ar: nested-dissection multifrontal structure (host analysis) */
    int64_t n_factor;                   /* kept nodes */
    const int64_t* perm;                /* [S*nx*ny] dense node -> factor index, -1 when not kept */
    int32_t n_fronts, n_levels;
    const int64_t* level_ptr;           /* [n_levels+1] into front_order */
    const int64_t* front_order;         /* [n_fronts] fronts sorted by height */
    const int64_t* own_start, *nown, *nbnd;      /* [n_fronts] */
    const int64_t* bnd_ptr, *bnd_idx;            /* CSR: boundary factor indices per front */
    const int64_t* child_ptr, *child_idx;        /* CSR: children per front */
    const int64_t* cmap_ptr, *cmap_idx;          /* per child entry: its boundary's rows in the parent front */
    const int64_t* panel_off, *upd_off, *vec_off;/* [n_fronts] element offsets */
    int64_t panel_total, upd_total, vec_total;
    const int64_t* ent_ptr;             /* [n_fronts+1] assembly entries per front */
    const int32_t* ent_row, *ent_col;   /* front row / own column */
    const int64_t* ent_s;               /* index of the S value */
    int64_t n_svalues;                  /* lower-triangle entries of S */
    int32_t n_table;                    /* per-frequency admittance table length */
    const int64_t* sterm_ptr;           /* [n_svalues+1] CSR: S value = sum coef * table[tab] */
    const int32_t* sterm_tab;
    const double* sterm_coef;
    /* A derived stack (PlaneStack.with_branches, peec.py:1871-1912): the last n_lowrank (0..64) branches are
     * left out of the S-term map, whose Schur structure is its base's; its operators come from
     * gt_operators_derive.  0 for every other geometry. */
    int32_t n_lowrank;
    /* Strips narrower than the pitch (PlaneStack._widths, peec.py:1732-1820); all zero / NULL when every strip
     * is full width.  n_override positions have their own S x S blocks of D^-1 in the admittance table, right
     * after the code blocks (before the capacitances); override_x / override_y: [(nx-1)*ny] / [nx*(ny-1)] the
     * block index of each strip position or -1.  The system product's corrections, per row q (n_narrow rows):
     * dense position narrow_pos, sheet narrow_sheet, resistance factor narrow_rdelta = 1/width - 1, self
     * inductance change narrow_dl (H) and mutual changes narrow_val (H) with the dense columns narrow_col of
     * entries narrow_ptr[q] .. narrow_ptr[q+1] (the side-by-side neighbours, M_near). */
    int32_t n_override;
    const int32_t* override_x;
    const int32_t* override_y;
    int64_t n_narrow;
    const int64_t* narrow_pos;
    const int32_t* narrow_sheet;
    const double* narrow_rdelta;
    const double* narrow_dl;
    const int64_t* narrow_ptr;
    const int64_t* narrow_col;
    const double* narrow_val;
    /* Face sheets of screened layers (PlaneStack._faces / _twins, peec.py:1658-1716): n_layers node layers
     * (0: as many as sheets) and each sheet's layer sheet_layer[n_sheets] (the lower faces of the n_twins split
     * layers follow the layers).  The V segment holds n_layers x nx x ny nodes.  Rows of the narrow list with
     * narrow_partner >= 0 add the face coupling z_mut(narrow_twin) * narrow_twfac * x[narrow_partner]; the
     * operators' zs then carry, per operator, the n_sheets sheet impedances followed by the n_twins couplings. */
    int32_t n_layers;
    const int32_t* sheet_layer;
    int32_t n_twins;
    const int64_t* narrow_partner;
    const int32_t* narrow_twin;
    const double* narrow_twfac;
    /* Resistance factors (PlaneStack.set_resistance_scale, peec.py:2199-2216), NULL when none: per row the real
     * part's extra factor of the strip's own impedance (narrow_rre = (scale - 1) / width) and of its face
     * coupling (narrow_twre). */
    const double* narrow_rre;
    const double* narrow_twre;
    /* Plane-pair capacitance of partly covered cells (PlaneStack.__init__'s per-cell facing area,
     * peec.py:1622-1637: C = c_per_area d^2 min(fill_upper, fill_lower)), NULL when every cell is whole: per cell
     * [n_pairs][nx][ny] of the C segment the covered share (> 0 where the cell has a capacitance); the cell's
     * impedance is the operator's zcap of its pair over the share and its D^-1 entry the table's times it. */
    const double* cap_fill;
} gt_geometry_desc;

typedef struct gt_solve_opts {
    double tol;             /* stop when ||b - K x|| <= tol * ||b|| in FP64 (peec.py:3098-3099) */
    int32_t restart;        /* inner GMRES cycle length */
    int32_t max_its;        /* total inner iterations allowed per column */
    double inner_tol;       /* relative residual reduction each inner FP32 cycle aims at */
    int32_t precision;      /* 0: FP32 inner GMRES + FP64 refinement, 1: all FP64 (plain drop-in), 2: as 0 with
                               the inner Krylov basis stored in FP16 (half the Gram-Schmidt traffic), 3: as 0 with
                               the preconditioner applied in FP64.  0 becomes 3 by itself when a column's
                               factorisation is stiff: a branch or capacitance admittance above 4096 times the
                               largest strip admittance (a near-short, whose current FP32 node potentials cannot
                               resolve), provided the FP64 sweeps fit its fronts; gt_memory counts what the
                               precision passed to it needs (pass 3 to plan a stiff solve) */
    int32_t max_outer;      /* refinement steps */
    double reorth;          /* DGKS: re-orthogonalise when ||w|| fell below reorth x its norm before the first
                               Gram-Schmidt pass (0.7: the reference's rule, peec.py:3156; 0: never) */
    int32_t outer_k;        /* FP64 outer GCR directions kept (each cycle's correction orthogonalised against
                               the previous ones; 1: a plain refinement step with the optimal step length) */
    int32_t use_guess;      /* nonzero: x holds each column's starting point on entry (the warm start x0 of
                               peec.py:2570-2578); the solve starts from r = b - K x0 in FP64 */
} gt_solve_opts;

/* Library version (major*10000 + minor*100 + patch). */
int gt_version(void);
/* Text of the calling thread's last failure ("" when none). */
const char* gt_last_error(void);
/* Number of CUDA devices visible (0 when none); the library needs one. */
int gt_device_count(void);
/* Kernels this library has launched since it was loaded (all threads). */
int64_t gt_launch_count(void);

/* Build a geometry on the current CUDA device (peec.py:1559-1593, gpu.py:617-666). */
int gt_geometry_create(const gt_geometry_desc* desc, gt_geometry** out);
void gt_geometry_free(gt_geometry* g);
/* Free the geometry's solve workspace (the Krylov bases and vectors sized for its largest solve so far); the next
 * solve allocates what it needs again.  For hosts that keep many geometries and solve them in turn under one
 * memory budget (the reference's memory gate, peec.py:1388-1501, releases solver memory between jobs). */
int gt_geometry_trim(gt_geometry* g);

/* Factorise the Schur complement at n_ops frequencies (peec.py:2345-2445, 2465-2511):
 * omega[n_ops]; zs[n_ops*(S + n_twins)] sheet impedances per square (then the face couplings, with face sheets); zcap[n_ops*n_pairs] and zbr[n_ops*n_branches]
 * the capacitance / branch impedances; table[n_ops*n_table] the admittance table D^-1 draws from. */
int gt_operators_create(gt_geometry* g, int32_t n_ops, const double* omega, const double* zs,
                        const double* zcap, const double* zbr, const double* table, gt_operators** out);
/* As gt_operators_create, with preconditioners shared between operators: factor_of[q] (0..n_ops-1) names the
 * operator whose Schur factorisation and D^-1 blocks precondition operator q; an operator so named must be its
 * own (factor_of[factor_of[q]] == factor_of[q]), and only those are factorised.  The system at q is q's own
 * (a borrowed preconditioner: PlaneStack.operator / _lend, peec.py:2227-2343).  factor_of NULL: every operator
 * its own. */
int gt_operators_create_shared(gt_geometry* g, int32_t n_ops, const double* omega, const double* zs,
                               const double* zcap, const double* zbr, const double* table, const int32_t* factor_of,
                               gt_operators** out);
/* As gt_operators_create_shared with flags.  GT_OPS_FP32_PANELS: keep only the FP32 copies of the factor panels
 * (column- and row-major, 16 bytes per entry instead of 48): the FP64 factor is made in temporary memory and
 * freed once converted, no FP64 row-major copy is made.  Such operators serve precision 0 and 2 solves and FP32
 * applications; precision 1 and 3, FP64 preconditioner applications and gt_operators_derive on them return
 * GT_INVALID_ARGUMENT.  A stiff set (see gt_solve_opts.precision) keeps its FP64 panels regardless.  For hosts
 * that keep many factorisations resident under a memory budget (the reference's memory gate and relief ladder,
 * peec.py:1388-1501, 2425-2430, trade factorisations for memory the same way). */
#define GT_OPS_FP32_PANELS 1
int gt_operators_create_ex(gt_geometry* g, int32_t n_ops, const double* omega, const double* zs,
                           const double* zcap, const double* zbr, const double* table, const int32_t* factor_of,
                           int32_t flags, gt_operators** out);
/* Operators of a derived geometry (n_lowrank > 0) from its base's (peec.py:2345-2377): operator q is the
 * base's operator q with the added branches, preconditioned by the base's factorisation of q plus the
 * Woodbury identity for the added branches (S' = S + U diag(1/z) U^T; only an n_lowrank x n_lowrank matrix
 * per factorisation is inverted).  Arguments as gt_operators_create for the derived geometry (zbr and table
 * with its branches), n_ops equal to the base's.  The base's factor panels are shared, not copied: free the
 * derived operators before the base's. */
int gt_operators_derive(gt_geometry* g, const gt_operators* base, int32_t n_ops, const double* omega,
                        const double* zs, const double* zcap, const double* zbr, const double* table,
                        gt_operators** out);
void gt_operators_free(gt_operators* ops);

/* Solve n_cols columns K x = rhs (peec.py:2560-2607): col_op[n_cols] the operator of each column,
 * rhs[n_cols*n_compact] complex in the reference's unknown order, x_out the same shape; its_out the inner
 * iterations, resid_out the final relative FP64 residual per column.  stream: a cudaStream_t or NULL.
 * Returns GT_NOT_CONVERGED when any column missed tol (its x is still the best found). */
int gt_solve(gt_geometry* g, gt_operators* ops, int32_t n_cols, const int32_t* col_op, const double* rhs,
             const gt_solve_opts* opts, double* x_out, int32_t* its_out, double* resid_out, void* stream);

/* Device memory of solves (the reference's memory gate, peec.py:1388-1501, gpu.py:593-605): *need the bytes a
 * gt_solve of n_cols columns with these options allocates (its workspace and the staging of the compact vectors),
 * *held those the geometry's workspace holds now (freed before a larger one is made, reused otherwise), *free_bytes
 * and *total_bytes the device's.  Any output pointer may be NULL. */
int gt_memory(gt_geometry* g, int32_t n_cols, const gt_solve_opts* opts, int64_t* need, int64_t* held,
              int64_t* free_bytes, int64_t* total_bytes);

/* The same with device-resident dense vectors: rhs_device / x_device are [n_cols*n_dense] complex128 in the
 * dense layout; nothing crosses to the host but the per-column scalars. */
int gt_solve_device(gt_geometry* g, gt_operators* ops, int32_t n_cols, const int32_t* col_op,
                    const void* rhs_device, const gt_solve_opts* opts, void* x_device, int32_t* its_out,
                    double* resid_out, void* stream);

/* Scatter compact (reference-order) complex vectors to the dense layout on the device and back. */
int gt_to_dense(gt_geometry* g, int32_t n_cols, const double* compact, void* dense_device, void* stream);
int gt_to_compact(gt_geometry* g, int32_t n_cols, const void* dense_device, double* compact, void* stream);

/* Single operator applications for parity tests, compact vectors in and out:
 * kind 0: system product K x (peec.py:3043-3062), 1: preconditioner M^-1 x (3064-3083),
 * 2: L_p product of the strip part (2115-2135); precision 0: FP32, 1: FP64. */
int gt_apply(gt_geometry* g, gt_operators* ops, int32_t kind, int32_t precision, int32_t n_cols,
             const int32_t* col_op, const double* x, double* y, void* stream);

/* Size of the fixed device scratch array gt_lp_product_noalloc uses (bytes). */
#define GT_LP_NOALLOC_SCRATCH_BYTES (32u << 20)

/* The L_p (partial-inductance) product of the strip currents of n_cols dense complex128 vectors
 * (x_device, n_cols * n_dense, the dense layout), written into the strip segments of y_device (its other
 * segments are left as they are), without allocating any device memory: for callers that may not allocate
 * while they compute (a process under a fixed device-memory budget, a latency-critical caller that cannot
 * afford cudaMalloc's device-wide synchronisation).  The FFT scratch comes from a fixed array of
 * GT_LP_NOALLOC_SCRATCH_BYTES held by every GPU that loads this library; n_cols beyond what it holds is
 * rejected with GT_INVALID_ARGUMENT.  The first call on a device looks the array's address up (make it before
 * any stream capture); calls whose kernels overlap on the GPU race on the shared array.  No counterpart in
 * the reference: it is an addition of this library. */
int gt_lp_product_noalloc(gt_geometry* g, int32_t n_cols, const void* x_device, void* y_device, void* stream);

/* psi of every strip (the flux per ampere of a signal path along it; peec.py:2615-2656 with
 * kernel.py:297-312), FP64 on the device, in the reference's strip order (x strips then y strips, the first
 * n_strips entries of the compact order).  sheet_z / sheet_t: [n_sheets] each sheet's face z (m) and copper
 * thickness (m); pitch in m; segments: [n_seg][8] rows (ax, ay, az, bx, by, bz, width, current) in host memory;
 * psi: [n_strips] host output.  Returns n_strips in *n_strips. */
int gt_strip_coupling(gt_geometry* g, const double* sheet_z, const double* sheet_t, double pitch, int32_t n_seg,
                      const double* segments, double* psi, int64_t* n_strips);

/* Outputs of dense FP64 device solutions x [n_cols][n_dense] (as gt_solve_device writes them), on the device.
 * gt_node_field: (Kx, Ky) at every node of every sheet in A/m per A (Solution.node_field, peec.py:1151-1203,
 * copper=False): each node averages the strips of each direction that touch it and carry current, over the
 * pitch; kx, ky: device [n_cols][n_sheets][nx][ny] complex128.
 * gt_moment: the plane's part of the magnetic moment m = 1/2 sum r x I dl (strips, plane-pair capacitances,
 * branches; PlaneStack.moment, peec.py:2668-2700) per column; the signal segments' own part is the caller's;
 * sheet_z: [n_sheets] host; m: [n_cols][3] complex128 host. */
int gt_node_field(gt_geometry* g, int32_t n_cols, const void* x_device, double pitch, void* kx_device,
                  void* ky_device, void* stream);
int gt_moment(gt_geometry* g, int32_t n_cols, const void* x_device, const double* sheet_z, double pitch, double* m,
              void* stream);

/* The real (P0/2+1) x (P1/2+1) quadrant of the spectrum of the partial-inductance kernel between square
 * strips of pitch d (m) on sheets dz (m) apart, over (2 n_axial - 1) x (2 n_lateral - 1) grid offsets wrapped
 * onto a P0 x P1 torus (peec.py:3276-3306, 3362-3371; kernel.py:170-176, 268-294), FP64 on the current
 * device.  near: [n_near][n_near] the tape-integrated values at the nearest offsets |axial|, |lateral| < n_near
 * (host); quad: host output, row-major [P0/2+1][P1/2+1].  P0, P1: 2^a or 3*2^a with a >= 3. */
int gt_kernel_spectrum(int32_t n_axial, int32_t n_lateral, double d, double dz, int32_t P0, int32_t P1,
                       const double* near, int32_t n_near, double* quad);

/* Per-kernel-family timing of the solves on this geometry, by CUDA events on the launch stream.
 * names == NULL and cap == -2: reset and switch timing on; cap == -3: the same, with each elimination level
 * of the triangular solves also timed as a family of its own ("fwd_f32.L<h>"); cap == -1: switch it off.
 * Otherwise fills
 * names (comma separated), ms (milliseconds), bytes (algorithmic bytes moved) and launches (timed
 * regions) per family, up to cap families, and returns their count. */
int gt_profile(gt_geometry* g, char* names, int32_t names_cap, double* ms, double* bytes, int32_t* launches,
               int32_t cap);

#ifdef __cplusplus
}
#endif
#endif /* GT_GB300_H */
