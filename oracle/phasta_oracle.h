/*
 * phasta_oracle.h -- CPU restatement (FP64) of PHASTA's compressible
 * matrix-free Newton-Krylov hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * GB300 kernels and the timed CPU baseline of the benchmark.  The product
 * (phasta_gb300) never links, loads or calls it.
 *
 * Parity status: the quadrature and shape-function tables are pinned against
 * the reference's own C sources (symtet.c, symtri.c, symhex.c, symwdg.c,
 * uniformP.c, newshape.cc) compiled in place; the Fortran routines are pinned
 * by golden vectors computed by the reference's own Fortran source, executed
 * through the Fortran-to-numpy translator in tests/golden.
 *
 * Array layouts are the reference's (Fortran column-major, node index
 * fastest):
 *   y, ac  (nshg, 5)   : y[k*nshg + n], global dof order (u, v, w, p, T)
 *   res    (nshg, 5)   : res[k*nshg + n], equation order (cont, mx, my, mz, energy)
 *   BDiag  (nshg, 5,5) : bd[(i + 5*j)*nshg + n]  for row i, column j (0-based)
 *   x      (nshg, 3)   : x[d*nshg + n]
 * Connectivity is 0-based.
 */
#ifndef PHASTA_ORACLE_H
#define PHASTA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* The COMMON-block values the hot path reads (common.h /mmatpar/, /timdat/,
 * /intdat/, /solpar/, /itrpar/, /precis/).  Filled by the caller. */
typedef struct {
    double Rgas, gamma, gamma1, pr;   /* gas constant, ratio of specific heats, gamma-1, Prandtl */
    double rmu;                       /* datmat(1,2,1): constant dynamic viscosity */
    double Dtgl, almi, alfi, gami;    /* 1/dt and generalized-alpha parameters */
    double dtsfct, taucfct, temper;   /* tau time constant, tau_C scale, energy tau scaling */
    int    itau, ivart, iremoveStabTimeTerm, Navier, ipord, EntropyPressure;
    int    Kspace, nGMRES, minIters;  /* GMRES controls */
    double etol, epsM;                /* Krylov tolerance, sqrt(machine eps) */
    double eGMRES;                    /* finite-difference interval (in/out) */
    int    iter, istep;               /* Newton iteration (1-based) and time step (0-based) */
    int    idiff;                     /* 0, or 1: global reconstruction of the diffusive flux */
    int    iDC;                       /* discontinuity capturing: 0 off, 1 DC-mallet, 2 quadratic, 3 min */
} or_common;

/* a block of boundary hexes or wedges (genbkb.f blocks; elmmfg.f:171-211): lcsyst 2 the hex with
 * its zeta = -1 quadrilateral face, 3 the wedge with its zeta = -1 triangle, 4 the wedge with its
 * s = 0 quadrilateral (face nodes 1, 4, 5, 2 in getbnodes' order, hierarchic.f:161-164) */
typedef struct {
    int lcsyst;
    int nelem;
    const int* ien;           /* nelem*nshl (8 for lcsyst 2, else 6) */
    const int* iBCB;          /* nelem*2 */
    const double* BCB;        /* nelem*nshlb*6 : BCB[(e*nshlb + n)*6 + k] */
} or_bnd_block;

typedef struct {
    int nshg;                 /* number of (stored) nodes */
    int nelem;                /* interior tets */
    const int* ien;           /* nelem*4, element-major (ien[4*e + a]) */
    int nblk;                 /* element blocks (<= 64 elements each) */
    const int* blk_start;     /* nblk+1 offsets into the element list */
    int ngrp;                 /* block groups: no two elements in a group share a node */
    const int* grp_start;     /* ngrp+1 offsets into the block list */
    const double* x;          /* (nshg,3) */
    int nbelem;               /* boundary tets (face nodes first) */
    const int* ienb;          /* nbelem*4 */
    const int* iBCB;          /* nbelem*2 : (flags, surface id) element-major */
    const double* BCB;        /* nbelem*3*6 : BCB[(e*3 + n)*6 + k] */
    const int* iBC;           /* nshg */
    const double* BC;         /* (nshg, ndofBC=6) column-major: BC[k*nshg + n] */
    const int* iper;          /* nshg, 0-based master (== n for non-periodic) */
    int nhex;                 /* interior linear hexes (lcsyst 2) */
    const int* ienh;          /* nhex*8, reference local node order */
    int nwedge;               /* interior linear wedges (lcsyst 3) */
    const int* ienw;          /* nwedge*6 */
    int nbblk;                /* blocks of boundary hexes and wedges */
    const or_bnd_block* bblk;
} or_mesh;

typedef struct {
    int    iKs;          /* Krylov iterations of the last cycle */
    int    lGMRES;       /* restarts done */
    int    ntotGM;       /* running GMRES iteration count (in/out) */
    double unorm0;       /* ||L^-1 R|| at entry */
    double echeck;       /* final |eBrg(iKs+1)| */
    double eGMRES;       /* FD interval used */
    double totres;       /* rstat measure sqrt(sum res^2)/nshg */
} or_solve_stats;

int or_make_groups(int nshg, int nelem, const int* ien, int bksiz, int* perm, int* blk_start,
                   int* nblk_out, int* grp_start, int max_grp);

/* quadrature/shape tables for linear tets (genint.f + genshp.f, p=1):
 * shp[q*4+a], shgl[(q*3+i)*4+a], Qwt[q]; boundary: shpb, shglb, Qwtb (3 qp) */
void or_tet_tables(double shp[16], double shgl[48], double Qwt[4],
                   double shpb[12], double shglb[36], double Qwtb[3]);

/* one element, e3.f: yl, ycl, acl (4,5) in element dof order (p,u,v,w,T),
 * xl (4,3); outputs rl, rml (4,5) and bdl (4,5,5) are ACCUMULATED. */
void or_e3(const or_common* c, int ires, int iprec,
           const double* yl, const double* ycl, const double* acl,
           const double* xl, double* rl, double* rml, double* bdl);

/* boundary quadrature/shape tables (genint.f, genshpb.f) of boundary topology lcsyst 2, 3 or 4:
 * shpb[q*nshl+a], shglb[(q*3+i)*nshl+a], Qwtb[q]; nshl, nshlb, ngaussb and the face nodes lnode
 * (0-based, getbnodes order) */
void or_btopo_tables(int lcsyst, double shpb[32], double shglb[96], double Qwtb[4], int* nshl, int* nshlb,
                     int* ngaussb, int lnode[4]);

/* quadrature/shape tables of topology lcsyst (1 tet, 2 hex, 3 wedge):
 * shp[q*nshl+a], shgl[(q*3+i)*nshl+a], Qwt[q] */
void or_topo_tables(int lcsyst, double shp[64], double shgl[192], double Qwt[8], int* nshl, int* ngauss);
/* one element of topology lcsyst, arrays (nshl,5)/(nshl,3)/(nshl,5,5) as in or_e3 */
void or_e3_topo(const or_common* c, int lcsyst, int ires, int iprec, const double* yl, const double* ycl,
                const double* acl, const double* xl, double* rl, double* rml, double* bdl);

/* one boundary element, e3b.f (ires in {1,3} adds rl) */
void or_e3b(const or_common* c, int ires, const double* yl, const int* iBCB,
            const double* BCB, const double* xlb, double* rl);

/* ElmMFG (elmmfg.f): res, rmes, BDiag over the mesh + boundary + BCs. */
void or_elmmfg(const or_common* c, const or_mesh* m, const double* y, const double* ac,
               double* res, double* rmes, double* bdiag, int iprec, int nthreads);

/* ItrRes (itrres.f): ADDS the modified residual of (yp, yc) into rmes, then bc3Res. */
void or_itrres(const or_common* c, const or_mesh* m, const double* yp, const double* yc,
               const double* ac, double* rmes, int iabres, int nthreads);

/* residual only (ires=1) over interior + boundary elements + bc3Res */
void or_elmres(const or_common* c, const or_mesh* m, const double* y, const double* ac,
               double* res, int nthreads);

void or_bc3res(const or_mesh* m, const double* y, double* res, const or_common* c);
void or_bc3bdg(const or_mesh* m, const double* y, double* bdiag, const or_common* c);
void or_itrbc(const or_mesh* m, double* y, double* ac, int ires, double Rgas);

/* i3LU (i3lu.f): code 0 LU_Fact, 1 forward, 2 backward, 3 product */
void or_i3lu(int nshg, double* bdiag, double* r, int code);
/* yshuffle: code 0 'old2new ', 1 'new2old ' (r is (nshg,5) column-major) */
void or_yshuffle(int nshg, double* r, int code);

/* SolMFG (solmfg.f): returns res (L^-1 R), BDiag (LU), Dy. c->eGMRES in/out. */
void or_solmfg(or_common* c, const or_mesh* m, const double* y, const double* ac,
               double* res, double* bdiag, double* Dy, or_solve_stats* st, int nthreads);

/* sparse solver (lhs = 1).  colm (nshg+1), rowp (nnz_tot) are 1-based as in the
 * reference; lhsK (25, nnz_tot) column-major: lhsK[25*k + 5*g + f] is entry (f, g)
 * of block k. */
/* genadj.f + asadj.f; returns -1 where the reference stops ("increase nnz") */
int or_genadj(const or_mesh* m, int nnz, int* colm, int* rowp, int* icnt);
/* ElmGMRs (elmgmr.f:280) with lhs = iprec = 1 */
void or_elmgmrs(const or_common* c, const or_mesh* m, const double* y, const double* ac, const int* colm,
                const int* rowp, int nnz_tot, double* res, double* bdiag, double* lhsK, int nthreads);
/* Spsi3pre (spsi3pre.f) with the i3LU factors in bd */
void or_spsi3pre(int nshg, const int* colm, const int* rowp, const double* bd, double* lhsK);
/* SparseAp (sparseap.f) then bc3per (bc3per.f): p <- lhsK p */
void or_sparseap(const or_mesh* m, const int* colm, const int* rowp, const double* lhsK, double* p);
/* SolGMRs (solgmr.f:480); st->lGMRES in: the COMMON lGMRES of the restart test */
void or_solgmrs(or_common* c, const or_mesh* m, const int* colm, const int* rowp, int nnz_tot,
                const double* y, const double* ac, double* res, double* bdiag, double* Dy, double* lhsK,
                or_solve_stats* st, int nthreads);

/* element-by-element solver (impl = 3x) on single-topology meshes.  EG is the reference's
 * EGmass(numel, nedof, nedof) column-major, elements in block order (tets in input order:
 * eid[e] = input id of the oracle's element e, NULL = identity; then hexes, wedges),
 * nedof = 5 x (nodes per element). */
void or_elmgmre(const or_common* c, const or_mesh* m, const int* eid, const double* y, const double* ac,
                double* res, double* bdiag, double* EG, int nthreads);
void or_i3pre(const or_mesh* m, const int* eid, const double* bd, double* EG);
/* Au1GMR (au1gmr.f) then bc3per: p <- sum_e EGmass_e p_e */
void or_au1gmr(const or_mesh* m, const int* eid, const double* EG, double* p);
void or_solgmre(or_common* c, const or_mesh* m, const int* eid, const double* y, const double* ac, double* res,
                double* bdiag, double* Dy, double* EG, or_solve_stats* st, int nthreads);

/* itrPC.f */
void or_itrpredict(const or_common* c, int nshg, const double* yold, const double* acold,
                   double* y, double* ac);
void or_itrcorrect(const or_common* c, int nshg, double* y, double* ac, const double* yold,
                   const double* acold, const double* Dy);
void or_itrupdate(const or_common* c, int nshg, double* yold, double* acold,
                  const double* y, const double* ac);

#ifdef __cplusplus
}
#endif
#endif
