/*
 * phgpu.h -- C ABI of the GB300-native drop-in for PHASTA's compressible
 * matrix-free Newton-Krylov hot path (one GPU, sm_103a).
 *
 * The entry points replace, with the same argument meaning, these reference
 * routines (paths within the PHASTA project):
 *
 *   phgpu_elmmfg     ElmMFG   phSolver/compressible/elmmfg.f:1-5
 *                    (interior AsIMFG/e3 + boundary AsBMFG/e3b + bc3Res + bc3BDg)
 *   phgpu_elmres     ElmMFG with iprec = 0 and no modified residual (res only)
 *   phgpu_itrres     ItrRes   phSolver/compressible/itrres.f:1-5 (adds into rmes)
 *   phgpu_i3lu       i3LU     phSolver/compressible/i3lu.f:1
 *   phgpu_solmfg     SolMFG   phSolver/compressible/solmfg.f:1-7
 *   phgpu_itrcorrect itrCorrect + itrBC  phSolver/compressible/itrPC.f:128, itrbc.f:1
 *   phgpu_newton     one flow solve of the itrdrv multi-corrector loop
 *                    (SolMFG + itrCorrect + itrBC, itrdrv.f:489-506, 596-598)
 *   phgpu_time_step  itrPredict + itrBC + nitr x phgpu_newton + itrUpdate + itrBC
 *                    (itrdrv.f:398-399, 427-634, 651-652)
 *
 * Host arrays keep the reference layout (Fortran column-major, node index
 * fastest) and dof orders:
 *   y, ac, yold, acold (nshg, 5): y[k*nshg + n], k over (u, v, w, p, T)
 *   res, rmes, Dy      (nshg, 5): r[k*nshg + n], k over (continuity, x-, y-, z-momentum, energy)
 *                                  = the (p, u, v, w, T) order of the element routines
 *   BDiag        (nshg, 5, 5)   : bd[(i + 5*j)*nshg + n]
 *   x            (nshg, 3)      : x[d*nshg + n]
 * Connectivity is 0-based.  The "_dev" suffix marks entry points that work on
 * the state already resident in the context's device memory.
 *
 * Every entry point returns a status code instead of stopping the program as
 * the reference's error()/tnanq do (common/error.f, tnanq.f); the message of
 * the last failure is available from phgpu_last_error().
 */
#ifndef PHGPU_H
#define PHGPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PHGPU_OK = 0,
    PHGPU_ERR_INVALID = 1,     /* bad argument or size */
    PHGPU_ERR_CUDA = 2,        /* CUDA runtime failure (no device, launch failure, ...) */
    PHGPU_ERR_NONFINITE = 3,   /* NaN/Inf in a residual or in the solution update (tnanq.f) */
    PHGPU_ERR_SINGULAR = 4,    /* zero or non-finite pivot in the 5x5 block LU */
    PHGPU_ERR_UNSUPPORTED = 5, /* option outside the implemented path */
    PHGPU_ERR_NOMEM = 6,       /* device allocation failed */
    PHGPU_ERR_TOO_LARGE = 7,   /* input larger than a fixed-size entry point accepts */
    PHGPU_ERR_IO = 8,          /* file could not be opened, read or written (phgpu_io.h) */
    PHGPU_ERR_NOTFOUND = 9     /* header key not found in a PHASTA file (phgpu_io.h) */
};

enum { PHGPU_FP64 = 0, PHGPU_MIXED = 1 };         /* precision */
/* Jacobian-vector product: finite-differenced (Au1MFG), linearized, the assembled tangent
 * of the sparse solver (SolGMRs, solgmr.f:480) or the stored element tangents of the
 * element-by-element solver (SolGMRe, solgmr.f:1) */
enum { PHGPU_AP_FD = 0, PHGPU_AP_LINEAR = 1, PHGPU_AP_SPARSE = 2, PHGPU_AP_EBE = 3 };
enum { PHGPU_RES_FP64 = 0, PHGPU_RES_GALERKIN64 = 1, PHGPU_RES_SPLITDF = 2 }; /* outer residual in mixed precision */
enum { PHGPU_LU_FACT = 0, PHGPU_LU_FORWARD = 1, PHGPU_LU_BACKWARD = 2, PHGPU_LU_PRODUCT = 3 };

/* The COMMON-block values the hot path reads (common.h), plus three options
 * of this implementation.  Field meanings follow the reference names. */
typedef struct {
    double Rgas, gamma, gamma1, pr;  /* mmatpar: gas constant, gamma, gamma-1, Prandtl */
    double rmu;                      /* datmat(1,2,1): constant viscosity (matflg(2)=0) */
    double Dtgl, almi, alfi, gami;   /* timdat: 1/dt and generalized-alpha factors */
    double dtsfct, taucfct, temper;  /* Tau Time Constant, Tau C Scale Factor, Temperature scaling */
    int itau;                        /* 0 (Diagonal-Shakib) is the implemented tau */
    int ivart;                       /* 2 = SUPG, 1 = Galerkin */
    int iremoveStabTimeTerm;
    int Navier;                      /* 1 = Navier-Stokes, 0 = Euler */
    int ipord;                       /* 1 = linear basis (implemented) */
    int EntropyPressure;
    int Kspace, nGMRES, minIters;    /* solpar */
    double etol;                     /* epstol(1) */
    double epsM;                     /* sqrt(machine epsilon), input.f:30 */
    double eGMRES;                   /* finite-difference interval (itrpar), in/out */
    int iter, istep;                 /* Newton iteration (1-based) and time step (0-based) */
    /* options of this implementation */
    int precision;                   /* PHGPU_FP64: reference arithmetic; PHGPU_MIXED: FP32
                                        assembly and Ap, FP64 outer residual, dots, Givens, LU */
    int ap_mode;                     /* PHGPU_AP_FD (Au1MFG), PHGPU_AP_LINEAR, PHGPU_AP_SPARSE or
                                        PHGPU_AP_EBE (the drivers then solve with SolGMRs or
                                        SolGMRe, lhs = 1) */
    int outer_residual;              /* mixed precision only: PHGPU_RES_FP64 (every term FP64),
                                        PHGPU_RES_GALERKIN64 (metrics, Euler flux and time term FP64;
                                        least-squares and viscous terms FP32) or PHGPU_RES_SPLITDF
                                        (no FP64 arithmetic: the Euler flux of each element's node-3
                                        state in double-float, its increment over the element and
                                        the other terms in FP32) */
    int idiff;                       /* 0, or 1: global reconstruction of the diffusive flux
                                        (elmmfg.f:56-111) whose divergence enters the residual's
                                        least-squares term */
    int no_graph;                    /* 0: each GMRES cycle of the linearized, sparse and element-by-
                                        element solvers runs as one CUDA graph (one conditional node
                                        per Krylov iteration, skipped once the cycle has converged);
                                        1: launched kernel by kernel with a host check per iteration */
    int iDC;                         /* discontinuity capturing (e3dc.f): 0 off, 1 DC-mallet,
                                        2 DC-quadratic, 3 DC-min; FP64 with the finite-difference
                                        product (ElmMFG, ItrRes, SolMFG) */
    int no_pipe;                     /* 0: the FP32 linearized product runs as a persistent kernel
                                        that stages the next mesh chunk with cp.async while it
                                        computes the current one; 1: one CTA per chunk */
    int precond;                     /* PHGPU_PRECOND_BDIAG: the reference's block-diagonal LU
                                        (i3lu.f); PHGPU_PRECOND_LEARNED: in addition the learned
                                        network as the right preconditioner of flexible GMRES
                                        (mixed precision, linearized product; see phgpu_net_*) */
} phgpu_config;

enum { PHGPU_PRECOND_BDIAG = 0, PHGPU_PRECOND_LEARNED = 1 };

/* Mesh and boundary-condition arrays (what the reference keeps in
 * pointer_data mien/mienb/miBCB/mBCB and in iBC/BC/iper). */
/* A block of boundary hexes or wedges (the reference's boundary element blocks of lcsyst 2, 3
 * and 4, genbkb.f; handled by AsBMFG/e3b, elmmfg.f:171-211): each element whole, in the
 * reference's local node order, with its boundary face where getbnodes (hierarchic.f:90-165)
 * looks for it:
 *   lcsyst 2  hex, the zeta = -1 quadrilateral: nodes 0-3 (nshl 8, nshlb 4)
 *   lcsyst 3  wedge, the zeta = -1 triangle: nodes 0-2 (nshl 6, nshlb 3)
 *   lcsyst 4  wedge, the s = 0 quadrilateral: nodes 0, 3, 4, 1 (nshl 6, nshlb 4)
 * BC values come per face node in that order.  The face's normal is the reference's: for
 * lcsyst 2 and 3, -(x1 - x0) x (x2 - x0); for lcsyst 4, dx/dr x dx/dzeta at each point. */
typedef struct {
    int lcsyst;
    int nelem;
    const int* ien;       /* nelem*nshl, element-major */
    const int* iBCB;      /* nelem*2: (flux bits, surface id) */
    const double* BCB;    /* nelem*nshlb*6: BCB[(e*nshlb + n)*6 + k] */
} phgpu_bnd_block;

typedef struct {
    int nshg;             /* nodes (periodic slaves are stored, as in the reference) */
    int nelem;            /* interior linear tets (lcsyst 1) */
    const int* ien;       /* nelem*4, element-major: ien[4*e + a] */
    const double* x;      /* (nshg, 3) */
    int nbelem;           /* boundary tets, boundary face = local nodes 0,1,2 */
    const int* ienb;      /* nbelem*4 */
    const int* iBCB;      /* nbelem*2: (flux bits as iBCB(:,1), surface id) */
    const double* BCB;    /* nbelem*3*6: BCB[(e*3 + n)*6 + k] as BCB(e, n, k) */
    const int* iBC;       /* nshg: BC bit codes (bit 1 T, bit 2 p, bits 3-5 velocity, bit 10 periodic) */
    const double* BC;     /* (nshg, 6) column-major, BC(:,k) */
    const int* iper;      /* nshg: periodic master (== n when not periodic) */
    /* further interior blocks (linear hexes and wedges, lcsyst 2 and 3), reference local node order */
    int nhex;             /* hexes */
    const int* ienh;      /* nhex*8 */
    int nwedge;           /* wedges */
    const int* ienw;      /* nwedge*6 */
    /* boundary hexes and wedges (the boundary tets are nbelem/ienb above) */
    int nbblk;
    const phgpu_bnd_block* bblk;
} phgpu_mesh;

typedef struct {
    int iKs;              /* Krylov iterations of the last GMRES cycle (solmfg.f:222) */
    int lGMRES;           /* restarts */
    int ntotGM;           /* running total of GMRES iterations (in/out) */
    int status;
    double unorm0;        /* ||L^-1 R|| before GMRES */
    double echeck;        /* final |eBrg(iKs+1)| */
    double eGMRES;        /* finite-difference interval used */
    double totres;        /* rstat measure: sqrt(sum res^2)/nshg of L^-1 R */
    double rnorm;         /* unpreconditioned FP64 ||R|| after BCs (nonlinear residual) */
    double t_assembly_ms, t_gmres_ms; /* device time of the phases, if timing is on */
    int net_its;          /* Krylov iterations of the learned flexible-GMRES cycle (0: none ran) */
    int net_fallback;     /* PHGPU_NET_*: how the solve used the learned preconditioner */
} phgpu_stats;

/* phgpu_stats.net_fallback */
enum {
    PHGPU_NET_USED = 0,      /* the learned cycle converged with fewer iterations, and in less
                                device time, than the reference block-diagonal solve needed */
    PHGPU_NET_FELL_BACK = 1, /* it did not (or produced a non-finite value): block-diagonal GMRES
                                cycles finished the solve from where it stopped */
    PHGPU_NET_PLAIN = 2      /* block-diagonal GMRES only: precond = BDIAG, no weights, the
                                reference count of a first solve, or the network switched off
                                after two failures in a row (or one more than twice as slow) */
};

typedef struct phgpu_ctx phgpu_ctx;

/* Reverse Cuthill-McKee order of the mesh's nodes (host only, no device needed): new_of_old[n]
 * is node n's number in the new order.  Nodes are adjacent when they share an interior element;
 * a periodic slave is adjacent to its master.  The caller renumbers its arrays with it before
 * phgpu_create (PHASTA's pre-processor does this before the solver reads the mesh); the optional
 * outputs give the graph's bandwidth max |i - j| over adjacent nodes before and after.
 * Deterministic (ties broken by node number); PHGPU_ERR_INVALID on a bad mesh. */
int phgpu_rcm_order(const phgpu_mesh* mesh, int* new_of_old, long long* bandwidth_before,
                    long long* bandwidth_after);

/* set-up: copies the mesh to the device, colours the elements; one GPU, one stream */
int phgpu_create(const phgpu_mesh* mesh, const phgpu_config* cfg, phgpu_ctx** out);
int phgpu_destroy(phgpu_ctx* ctx);
int phgpu_set_config(phgpu_ctx* ctx, const phgpu_config* cfg);
int phgpu_get_config(phgpu_ctx* ctx, phgpu_config* cfg);
const char* phgpu_last_error(phgpu_ctx* ctx);
void* phgpu_stream(phgpu_ctx* ctx);        /* the cudaStream_t every kernel runs on */
int phgpu_num_colors(phgpu_ctx* ctx);
long long phgpu_kernel_launches(phgpu_ctx* ctx); /* kernels launched since create */
/* GMRES cycles run as one CUDA graph since create (config no_graph = 0), or -1 when the
 * graph could not be built (phgpu_last_error then gives the reason; cycles run kernel by kernel) */
long long phgpu_graph_cycles(phgpu_ctx* ctx);
/* time steps run as one CUDA graph since create, or -1 when the graph could not be built
 * (phgpu_last_error gives the reason; steps are then launched kernel by kernel).  With
 * no_graph = 0, phgpu_time_step(_dev) of the mixed-precision block-diagonal matrix-free solver
 * (also with precond = PHGPU_PRECOND_LEARNED while the network is off or has no weights)
 * with nGMRES = 1 and nitr <= 16 runs itrPredict, the nitr Newton iterations (assembly, LU,
 * the GMRES cycle as conditional nodes opened from the device, back substitution, itrCorrect,
 * itrBC) and itrUpdate as one graph with one host read of the statistics: the same kernels in
 * the same order as kernel by kernel, so the state is bitwise the same; phgpu_stats then has
 * no phase timings (t_assembly_ms = t_gmres_ms = 0), and after a SINGULAR or NONFINITE status
 * the state of that step is undefined. */
long long phgpu_step_graphs(phgpu_ctx* ctx);

/* Autotuned register/occupancy variants of the two pipelined element sweeps of the mixed-precision
 * matrix-free solver: the linearized product (compiled for at least 3 or 4 resident CTAs per SM)
 * and the double-float split outer residual (2, 3 or 4).  Before its first mixed-precision
 * linearized solve or graph-captured time step, a context times each variant on its own mesh
 * and state (a warm-up and three timed sweeps each, CUDA events) and keeps the fastest when it
 * beats the compiled-in default by more than 5%, for the context's lifetime; on a mesh whose
 * default linearized product takes less than 0.5 ms the defaults stay untimed beyond it.  The variants are
 * the same arithmetic compiled under different register budgets: each is deterministic, and
 * they agree with one another to FP32 rounding (the compiler may fuse multiplies and adds
 * differently), not bit for bit.
 * phgpu_set_tuning forces a choice (lin_minb 3 or 4, ress_minb 2, 3 or 4), or with (0, 0)
 * returns to the compiled-in defaults and tunes again at the next solve, or with (-1, -1) does
 * so timing every variant whatever the mesh size.
 * phgpu_tuning gives the current choice and, in ms[5], the mean time of each variant in ms
 * (linearized product 3, 4; split residual 2, 3, 4; -1 when not timed); it returns 0 while
 * untuned, 1 when tuned, 2 when forced. */
int phgpu_set_tuning(phgpu_ctx* ctx, int lin_minb, int ress_minb);
int phgpu_tuning(phgpu_ctx* ctx, int* lin_minb, int* ress_minb, double* ms);

/* new values BC(nshg, 6) of the Dirichlet constraints (the iBC bits of phgpu_create stay): the
 * reference passes BC to every ElmMFG/SolMFG call (elmmfg.f:1-5, solmfg.f:1-7) */
int phgpu_set_bc(phgpu_ctx* ctx, const double* BC);

/* ElmMFG: res, rmes, BDiag (BDiag only when iprec != 0) */
int phgpu_elmmfg(phgpu_ctx* ctx, const double* y, const double* ac,
                 double* res, double* rmes, double* bdiag, int iprec);
/* residual only (ires = 1) with boundary faces and bc3Res */
int phgpu_elmres(phgpu_ctx* ctx, const double* y, const double* ac, double* res);
/* ItrRes: rmes += Rmod(yp; yc), then bc3Res */
int phgpu_itrres(phgpu_ctx* ctx, const double* yp, const double* yc, const double* ac,
                 double* rmes);
/* i3LU on host arrays */
int phgpu_i3lu(phgpu_ctx* ctx, double* bdiag, double* r, int code);
/* SolMFG: outputs res = L^-1 R, bdiag = LU factors, Dy (undefined when the status is
 * PHGPU_ERR_NONFINITE: a GMRES cycle run as a CUDA graph updates Dy before the host sees the flag) */
int phgpu_solmfg(phgpu_ctx* ctx, const double* y, const double* ac,
                 double* res, double* bdiag, double* Dy, phgpu_stats* st);
/* itrCorrect + itrBC on host arrays */
int phgpu_itrcorrect(phgpu_ctx* ctx, double* y, double* ac, const double* yold,
                     const double* acold, const double* Dy);
/* one multi-corrector flow solve on host arrays (y, ac updated in place) */
int phgpu_newton(phgpu_ctx* ctx, double* y, double* ac, const double* yold,
                 const double* acold, phgpu_stats* st);
/* one time step: yold/acold updated in place, y/ac returned */
int phgpu_time_step(phgpu_ctx* ctx, double* yold, double* acold, double* y, double* ac,
                    int nitr, phgpu_stats* st);

/* ---- sparse solver: the reference's impl = 1x path (lhs = 1, itrdrv.f:452-488) ----
 * lhsK is the reference's lhsK(25, nnz_tot) (FP64): block k is 25 contiguous values with
 * entry (f, g) of the 5x5 block at 25*k + 5*g + f (row f = equation, column g = dof);
 * the blocks follow genadj's colm/rowp, rows by node and columns ascending. */
/* genadj (genadj.f:1, asadj.f:1) on the host, no context or GPU needed: colm (nshg+1) and
 * rowp (room for nnz*nshg) 1-based as in the reference, *icnt = nnz_tot.  Returns
 * PHGPU_ERR_TOO_LARGE where the reference stops (a row of more than 15*nnz nodes, or more
 * than nnz*nshg blocks), PHGPU_ERR_INVALID for a node index out of range. */
int phgpu_genadj(const phgpu_mesh* mesh, int nnz, int* colm, int* rowp, int* icnt);
/* nnz_tot of the context's mesh (the first sparse call builds the device structure) */
int phgpu_nnz_tot(phgpu_ctx* ctx, int* nnz_tot);
/* ElmGMRs (elmgmr.f:280) with lhs = 1, iprec = 1, FP64: res, BDiag and lhsK */
int phgpu_elmgmrs(phgpu_ctx* ctx, const double* y, const double* ac, double* res, double* bdiag,
                  double* lhsK);
/* Spsi3pre (spsi3pre.f:1) on host arrays; bdiag holds the i3LU factors */
int phgpu_spsi3pre(phgpu_ctx* ctx, const double* bdiag, double* lhsK);
/* SparseAp (sparseap.f:1) then bc3per (bc3per.f:1), as SolGMRs applies them: p <- lhsK p */
int phgpu_sparseap(phgpu_ctx* ctx, const double* lhsK, double* p);
/* SolGMRs (solgmr.f:480) in the configured precision: lhs = 1 assembles BDiag and the tangent
 * (iprec = lhs, itrdrv.f:456-457); lhs = 0 reuses the factored BDiag and the preconditioned
 * tangent of the last lhs = 1 call (PHGPU_ERR_INVALID if there is none).  Outputs as
 * phgpu_solmfg, plus the preconditioned tangent in lhsK (FP64 solves; may be NULL).
 * st->lGMRES on entry is the COMMON lGMRES that SolGMRs' restart test reads
 * (solgmr.f:528, never set by SolGMRs itself); on return, the cycles done less one. */
int phgpu_solgmrs(phgpu_ctx* ctx, const double* y, const double* ac, int lhs, double* res,
                  double* bdiag, double* Dy, double* lhsK, phgpu_stats* st);

/* ---- element-by-element solver: the reference's impl = 3x path (itrdrv.f:507-526) ----
 * Only for meshes of one element topology (all tets, all hexes or all wedges): the
 * reference's i3pre gathers BDiag through a section of its (numel, nshape, 5, 5) array into
 * a (npro, nshl, 25) dummy, which scrambles the blocks of elements smaller than the largest
 * one; mixed meshes return PHGPU_ERR_UNSUPPORTED.  EGmass is the reference's
 * EGmass(numel, nedof, nedof) (FP64, column-major, elements in input order, nedof = 5 x
 * nodes per element). */
/* ElmGMRe (elmgmr.f:1) with lhs = 1, iprec = 1: res, BDiag and EGmass after bc3LHS */
int phgpu_elmgmre(phgpu_ctx* ctx, const double* y, const double* ac, double* res, double* bdiag,
                  double* EGmass);
/* i3pre (i3pre.f:1) on host arrays; bdiag holds the i3LU factors */
int phgpu_i3pre(phgpu_ctx* ctx, const double* bdiag, double* EGmass);
/* Au1GMR (au1gmr.f:1) then bc3per (bc3per.f:1), as SolGMRe applies them: p <- sum_e EGmass_e p */
int phgpu_au1gmr(phgpu_ctx* ctx, const double* EGmass, double* p);
/* SolGMRe (solgmr.f:1) in the configured precision; outputs as phgpu_solmfg, plus the
 * preconditioned EGmass (FP64 solves; may be NULL) */
int phgpu_solgmre(phgpu_ctx* ctx, const double* y, const double* ac, double* res, double* bdiag,
                  double* Dy, double* EGmass, phgpu_stats* st);

/* device-resident state (no host traffic inside) */
int phgpu_upload_state(phgpu_ctx* ctx, const double* y, const double* ac,
                       const double* yold, const double* acold);
int phgpu_download_state(phgpu_ctx* ctx, double* y, double* ac, double* yold, double* acold);
int phgpu_newton_dev(phgpu_ctx* ctx, phgpu_stats* st);
int phgpu_time_step_dev(phgpu_ctx* ctx, int nitr, phgpu_stats* st);
/* nonlinear residual ||R(y)|| (FP64, unpreconditioned, after BCs) of the resident state */
int phgpu_residual_norm_dev(phgpu_ctx* ctx, double* rnorm);
/* one element sweep of the resident state (timing probe of the hot kernels): 0 FP64 residual,
 * 1 FP64 modified residual, 2 FP32 linearized product, 3 FP32 block diagonal, 4 FP64 block
 * diagonal + residuals, 5 FP32 copies of the state, 6 FP64-Galerkin residual, 7 double-float
 * split residual, 8 hi/lo float copies of the state, 9 FP32 assembled tangent, 10 FP32
 * block-sparse product, 11 FP64 assembled tangent, 12 FP64 block-sparse product (9-12 use the
 * sparse solver's structure; 10 and 12 multiply whatever tangent 9 and 11 left), 13 FP32
 * element tangents stored per element, 14 FP32 element-by-element product (13-14: mixed
 * precision context, one element topology), 17 one application of the learned preconditioner
 * (weights set, after a mixed-precision solve), 18 its context features */
int phgpu_sweep_dev(phgpu_ctx* ctx, int which);

/* ---- learned preconditioner (no counterpart in the reference) --------------------------
 * A message-passing network over the mesh edges maps a Krylov vector v of the block-diagonal
 * preconditioned operator L^-1 J U^-1 (the operator SolMFG's loop multiplies by, au1mfg.f:57-83)
 * to z = P(v) ~ (L^-1 J U^-1)^-1 v; with precond = PHGPU_PRECOND_LEARNED the GMRES cycle of
 * solmfg.f:221-340 becomes flexible GMRES whose Krylov iteration j multiplies z_j = P(v_j) and
 * whose solution is sum_j y_j z_j.  The block-diagonal GMRES of the reference is the fallback:
 * the first solve of a context (and the first after new weights) runs it to set the reference:
 * its Krylov iterations and its device time per iteration.  Later solves cap the learned cycle one
 * iteration below that count; a learned cycle fails when it does not converge within the cap,
 * is not finite, or takes longer on the device than the reference iterations it replaces.  A
 * failed cycle is finished by block-diagonal cycles from where it stopped (nGMRES more cycles);
 * two failures in a row, or one learned cycle that takes more than twice the time of the
 * reference iterations it replaces, switch the network off until new weights are set.  The
 * network: encoder 48 -> 64, three edge
 * message-passing layers (hidden width 64), decoder 64 -> 5; BF16 GEMM operands with FP32
 * accumulation on the tensor cores, FP32 master weights.  Input per node: the direction (5), the
 * node's factored BDiag block (25, over their RMS), its state (5) and an active flag.
 * Weights are one FP32 array of PHGPU_NET_NPARAM values in this order (row-major matrices):
 *   W_e[64][48] b_e[64], then per layer l = 0..2: W_p[64][64] W_q[64][64] b_m[64] C[64][3]
 *   W_u[64][128] b_u[64], then W_d[5][64] b_d[5] alpha[5] beta[5]
 * (alpha, beta: per-dof input and output scales, set from the training pairs).
 * Host vectors v, t, z use the layout of res (nshg, 5). */
#define PHGPU_NET_NPARAM 53583
#define PHGPU_NET_NTRAIN 53573   /* trained values: all but alpha and beta */
typedef struct {
    int epochs;                      /* passes over the collected pairs */
    int npairs;                      /* pairs used (<= collected; 0: all) */
    float lr, beta1, beta2, eps;     /* Adam */
    float clip;                      /* global gradient-norm clip (0: none) */
    unsigned seed;                   /* pair order of each epoch */
    int renormalize;                 /* 1: set alpha and beta from the pairs first */
} phgpu_net_train_config;
typedef struct {
    double loss_first, loss_last;    /* mean loss of the first and of the last epoch */
    double ms;                       /* device time of the training */
    long long steps;
} phgpu_net_train_stats;
/* weights (copied); resets the fallback state */
int phgpu_net_set_weights(phgpu_ctx* ctx, const float* w, int n);
int phgpu_net_get_weights(phgpu_ctx* ctx, float* w, int n);
/* the edge graph: nstart (nshg+1), nbr (room for cap; 26-bit neighbour | shift code << 26,
 * code bits 2d..2d+1 = 1: +L_d, 2: -L_d), geo = {L_x, L_y, L_z, 1/hbar}; *nnz = edges */
int phgpu_net_graph(phgpu_ctx* ctx, int* nstart, unsigned* nbr, long long cap, long long* nnz, float* geo);
/* solves with precond = PHGPU_PRECOND_LEARNED since create, by outcome: counts[0] learned
 * cycle used, [1] fell back, [2] block-diagonal only; counts[3] = 1 while the network is off */
int phgpu_net_usage(phgpu_ctx* ctx, long long* counts);
/* context features of the resident state and FP32 factored BDiag (after a mixed-precision
 * solve): out (nshg, 32) as floats, may be NULL (computes them only) */
int phgpu_net_features(phgpu_ctx* ctx, float* out);
/* z = P(v) with the current features; hidden (4 x nshg x 64: h0..h3) and out (nshg x 8,
 * decoder outputs) may be NULL */
int phgpu_net_apply(phgpu_ctx* ctx, const double* v, double* z, float* hidden, float* out);
/* training loss and gradient (PHGPU_NET_NPARAM floats, alpha/beta entries 0) of one pair */
int phgpu_net_loss_grad(phgpu_ctx* ctx, const double* v, const double* t, double* loss, float* grad);
/* training pairs: room for cap pairs (frees the old set) */
int phgpu_net_pairs(phgpu_ctx* ctx, int cap);
/* after a mixed-precision block-diagonal solve (phgpu_solmfg): store pair `slot` from u = the
 * solve's Krylov-space solution U Dy (which = 0) or Krylov vector u_which of its last cycle
 * (1 <= which <= the cycle's iterations + 1): v = A~ u / ||A~ u||, t = u / ||A~ u|| (A~ t = v
 * exactly), with the current context features */
int phgpu_net_collect(phgpu_ctx* ctx, int slot, int which);
/* Adam over the collected pairs, one pair per step, on the GPU */
int phgpu_net_train(phgpu_ctx* ctx, const phgpu_net_train_config* cfg, phgpu_net_train_stats* out);

/* Largest 5*nshg that phgpu_rstat_noalloc accepts (33,554,432 values, nshg <= 6,710,886). */
#define PHGPU_RSTAT_NOALLOC_MAX_N 33554432
/* No counterpart in the reference: an allocation-free form of the residual
 * statistic that phgpu_solmfg reports as phgpu_stats.totres,
 * *totres = sqrt(sum_k res[k]^2) / nshg over the 5*nshg values of res.
 *
 * For callers that cannot allocate device memory -- a host code whose device
 * memory is all owned by its own pool or another framework's allocator, or a
 * phase that must not grow the device footprint or take the device-wide
 * synchronisation that cudaMalloc/cudaFree can imply.  It needs no context.
 * res and totres are DEVICE pointers owned by the caller; the call is
 * asynchronous on `stream` (a cudaStream_t, NULL = legacy default stream).
 * Its working storage is a fixed 128 KiB static device array inside the
 * library, held by every GPU that loads the library until the process exits;
 * it calls no cudaMalloc, cudaFree or other allocating routine.
 *   - The first call on a device looks up that array's device address
 *     (cudaGetSymbolAddress, with that device current) and caches it; make
 *     that first call before any stream capture.  A cudaDeviceReset of that
 *     device invalidates the cached address: do not call this entry point on
 *     it again in the same process after a reset.
 *   - `stream` must belong to the current device (PHGPU_ERR_INVALID otherwise).
 *   - Returns PHGPU_ERR_TOO_LARGE when 5*nshg > PHGPU_RSTAT_NOALLOC_MAX_N,
 *     PHGPU_ERR_INVALID for null pointers or nshg <= 0, PHGPU_ERR_CUDA when
 *     the address look-up or the launch fails.
 *   - Every call shares the one array: calls that can overlap on the GPU
 *     (concurrent streams, several host threads) race and give wrong results;
 *     serialise them on one stream.  Each call clears the array's completion
 *     counter itself, so no zeroing is required of the caller. */
int phgpu_rstat_noalloc(const double* res, int nshg, double* totres, void* stream);

/* Self-test of the bounded wait that guards every bulk copy of the pipelined sweeps (no context
 * needed; current device): one CTA arms an mbarrier that expects two arrivals, gives it one, and
 * waits at most `tries` times (1 .. 524,288, the sweeps' own limit: about 2 s, at about 4 us per
 * try on a GB300); *status receives 8 when the
 * wait gave up (the value a sweep sets in its error word before it ends), 0 if the phase
 * completed.  PHGPU_ERR_INVALID for a null status or tries out of range. */
int phgpu_selftest_wait_limit(int tries, int* status);

#ifdef __cplusplus
}
#endif
#endif
