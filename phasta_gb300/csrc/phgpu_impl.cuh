// phgpu_impl.cuh -- internal declarations of the GB300 implementation of the
// compressible Newton-Krylov hot path.  Device data layout:
//   nodal vectors  [node][5] in element dof order (p, u, v, w, T) / equation order
//   BDiag          [node][25], row-major 5x5 block (bd[n*25 + 5*i + j] = BDiag(n, i, j))
//   coordinates    [node][3]
//   connectivity   int4 per element, elements sorted by colour (no two elements
//                  of one colour share a stored node, so scatters are plain
//                  read-modify-writes, deterministic and atomic-free)
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/phgpu.h"

namespace phgpu {

constexpr int kBlock = 128;          // threads per block of the boundary kernel
constexpr int kChunk = 128;          // elements per chunk (one CTA per chunk)
constexpr int kRedBlocks = 4 * 152;  // fixed grid of the reductions (deterministic order)
constexpr int kRedThreads = 256;

// Physics constants of one assembly, derived from phgpu_config (passed by value).
template <typename R>
struct Phys {
    R Rgas, rRgas;       // R and 1/R
    R cv, cp;            // R/(gamma-1), R*gamma/(gamma-1)
    R rmu, rlm, rlm2mu, con, rlmpmu;  // viscosity, lambda, lambda+2mu, conductivity, lambda+mu
    R fct1;              // almi/gami/alfi*Dtgl
    R dts2;              // (2*dtsfct*Dtgl)^2  (0 if the time term is removed)
    R fmu2;              // 36*mu^2
    R taucfct, rtempcv;  // tau_C scale, temper/cv
    R epsM;              // sqrt(machine epsilon): the DC factor's guard (e3dc.f:260)
    R rdts, celt, temper;  // itau = 1: 1/(Dtgl dtsfct), the diffusive correction 2/3, temper
    int navier, supg;
    int idc;             // discontinuity capturing (FP64 residual kernels only)
    int itau;            // 0 Diagonal-Shakib, 1 Diagonal-Franca (FP64 kernels only)
};

// quadrature/shape tables for linear tets (host-computed, read-only in constant memory)
struct TetTables {
    double shp[4][4];    // [q][a]
    double Qwt[4];
    double shpb[3][4];
    double Qwtb[3];
};

// quadrature and shape tables of one element topology (linear basis, up to 8 points/nodes)
struct TopoTabD {
    double shp[8][8];      // [q][a]
    double shgl[8][3][8];  // [q][i][a] parent-coordinate derivatives
    double qwt[8];
};
struct TopoTabF {
    float shp[8][8];
    float shgl[8][3][8];
    float qwt[8];
};
// t[0] hex (lcsyst 2), t[1] wedge (lcsyst 3), t[2] tet (lcsyst 1)
void topo_tables_host(TopoTabD* t);

// block-sparse tangent of the sparse solver (lhs = 1), built on the first call that needs it
struct SparseCtx {
    bool ready = false;
    int nnzb = 0;                 // nnz_tot: 5x5 blocks
    std::vector<int> colm, rowp;  // the reference's genadj arrays (1-based)
    int* d_rs = nullptr;          // N+1 row starts (0-based)
    int* d_bcol = nullptr;        // nnzb column node
    int* d_bcolp = nullptr;       // nnzb iper(column node): SparseAp's periodic gather
    int* d_brow = nullptr;        // nnzb row node
    int* d_ient = nullptr;        // tets in tangent colour order (4 per element)
    std::vector<int> tcol_start;  // tet colours of the tangent
    int* d_tmap = nullptr;        // block index of (element, a, b): 16 per tet
    int* d_hmap = nullptr;        // 64 per hex (d_ienh order)
    int* d_wmap = nullptr;        // 36 per wedge (d_ienw order)
    double* d_lhsK = nullptr;     // 25 * nnzb, the reference's lhsK(25, nnz_tot) layout
    float* d_lhsKf = nullptr;     // FP32 tangent of the mixed-precision solve
    int have = -1;                // precision of the preconditioned tangent kept from the last lhs = 1 solve
    // element colouring of the tet tangent (shared with the element-by-element solver)
    bool tan_ready = false;
    std::vector<int> torder;      // tangent position -> input tet
    std::vector<int> h_ient;      // tets in tangent order (host copy of d_ient)
    // element-by-element solver: per element its NEN x NEN blocks (25 values, entry (f, g) at
    // 5 g + f), elements in tangent order (tets), d_ienh order (hexes) or d_ienw order (wedges)
    size_t eg_blocks = 0;
    double* d_EG = nullptr;
    float* d_EGf = nullptr;
};

// The GMRES cycle as one CUDA graph: one conditional (if) node per Krylov iteration whose
// body is that iteration's product, Gram-Schmidt and Givens kernels; the Givens kernel of
// iteration i opens node i+1 unless the cycle has converged.  Rebuilt when the options or
// the operator it was captured with change.
struct CycleGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<long long> launches;  // kernels in the body of iteration i
    phgpu_config key{};
    int vsize = 0, min_iters = 0;
    int lin_minb = 0;                 // the linearized-product variant fixed in the graph
    const void* lhs = nullptr;
    bool disabled = false;            // a graph call failed: cycles are launched kernel by kernel
    long long runs = 0;               // cycles run as a graph
    std::string why;
};

// A whole time step (itrPredict + itrBC, nitr Newton iterations, itrUpdate + itrBC) as one CUDA
// graph, for the mixed-precision block-diagonal matrix-free solve with one GMRES cycle: the
// assembly, the LU, the cycle (one conditional node per Krylov iteration, opened from the
// device) and the update are launched from the graph; the norms and the cycle's decisions stay
// on the device, and the statistics of every Newton iteration come back in one read.
// a block of boundary hexes or wedges on the device, its elements in colour order
struct BndBlockDev {
    int lcsyst = 0, nelem = 0, nshl = 0, nshlb = 0;
    int* d_ien = nullptr;      // nelem*nshl
    int* d_ibcb = nullptr;     // nelem*2
    double* d_bcb = nullptr;   // nelem*nshlb*6
    std::vector<int> col_start;
};

struct StepGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    phgpu_config key{};
    int nitr = 0;
    int lin_minb = 0, ress_minb = 0;  // the sweep variants fixed in the graph
    long long fixed_launches = 0;     // kernels outside the Krylov iterations
    std::vector<long long> body_launches;  // kernels of Krylov iteration i (1-based)
    bool disabled = false;
    std::string why;
    long long runs = 0;
    cudaStream_t aux = nullptr;       // the stream the Krylov iteration bodies are captured on
    double* d_stats = nullptr;        // per Newton iteration (8 values, see k_step_record)
};
constexpr int kStepGraphMaxNitr = 16;

// The learned right preconditioner of flexible GMRES (learn.cu): the mesh-edge graph of the
// message-passing network, its weights, per-solve context features, activation buffers,
// the preconditioned Krylov basis Z, the training set and the fallback state.
struct NetTrain {
    int cap = 0, npairs = 0;              // training pairs allocated / collected
    float* d_pv = nullptr;                // cap x 5N: input directions v (unit norm)
    float* d_pt = nullptr;                // cap x 5N: targets t
    __nv_bfloat16* d_pctx = nullptr;      // cap x 32N: context features of each pair
    // activations kept by the training forward for the backward
    __nv_bfloat16* d_hs = nullptr;        // 4 x 64N: h0..h3
    __nv_bfloat16* d_ps = nullptr;        // 3 x 64N: P of each layer
    __nv_bfloat16* d_as = nullptr;        // 3 x 64N: aggregated messages
    float* d_qs = nullptr;                // 3 x 64N: Q of each layer
    float* d_us = nullptr;                // 3 x 64N: update pre-activations
    float* d_out = nullptr;               // 8N: decoder outputs
    float* d_dh = nullptr;                // 64N: gradient of the hidden state
    float* d_dms = nullptr;               // 64N: gradient of the mean message
    __nv_bfloat16* d_dqp = nullptr;       // 128N: gradients of Q and P (bf16 GEMM operands)
    float* d_part = nullptr;              // grid x (NPARAM + 1) per-CTA partial gradients and loss
    float* d_grad = nullptr;              // NPARAM
    float* d_m = nullptr;                 // Adam moments
    float* d_v = nullptr;
    double* d_scal = nullptr;             // [0] grad norm^2, [1..] per-step losses
    int scal_cap = 0;
    int grid = 0;                         // CTAs of the training kernels
    long long step = 0;                   // Adam steps taken
};
struct NetCtx {
    bool graph = false;
    bool attrs_set = false;               // the kernels' shared-memory limits, on this context's device
    long long nnz = 0;
    int* d_nstart = nullptr;              // N+1 CSR row starts
    unsigned* d_nbr = nullptr;            // neighbour | periodic shift code << 26
    unsigned char* d_act = nullptr;       // 1: node the network corrects
    float4* d_x4 = nullptr;               // coordinates (FP32, padded to 16 bytes)
    int nact = 0;
    float L[3] = {0.f, 0.f, 0.f};         // periods of the translational periodicity
    float rh = 1.f;                       // 1 / mean edge length
    double hbar = 1.0;
    float* d_w = nullptr;                 // FP32 master weights (NPARAM)
    bool have_w = false;
    __nv_bfloat16* d_ctx = nullptr;       // 32N context features of the current solve
    float* d_stat = nullptr;              // normalisation of the context features
    double* d_spart = nullptr;            // their partial sums
    __nv_bfloat16* d_h = nullptr;         // 64N hidden state (inference, updated in place)
    __nv_bfloat16* d_P0 = nullptr;        // 64N message projections (ping-pong)
    __nv_bfloat16* d_P1 = nullptr;
    float* d_Z = nullptr;                 // Kspace x ldU preconditioned Krylov vectors
    int grid_enc = 1, grid_mp = 1;        // persistent grids of the inference kernels
    // fallback: Krylov iterations of the last block-diagonal solve (-1: none yet), consecutive
    // learned cycles that did not converge within fewer iterations, and the switch they throw
    int its_ref = -1, fails = 0;
    bool disabled = false;
    double ms_ref_iter = 0.0;             // device time per Krylov iteration of that solve
    double ms_last = 0.0;                 // device time of the last learned cycle
    long long n_used = 0, n_fell_back = 0, n_plain = 0;  // solves with precond = LEARNED, by outcome
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    NetTrain tr;
};

struct Ctx {
    int N = 0, E = 0, Eb = 0;
    phgpu_config cfg{};
    cudaStream_t stream = nullptr;
    int device = 0;
    std::string err;
    long long launches = 0;

    // element colouring
    std::vector<int> col_start;   // ncol+1 (interior)
    std::vector<int> bcol_start;  // boundary
    std::vector<BndBlockDev> bblk;  // boundary hexes and wedges (boundary.cu)
    int4* d_ien = nullptr;        // E (chunk order)
    // hex and wedge blocks (colour order)
    int nhex = 0, nwedge = 0;
    int* d_ienh = nullptr;        // nhex*8
    int* d_ienw = nullptr;        // nwedge*6
    std::vector<int> hcol_start, wcol_start;
    std::vector<int> horder, worder;  // colour position -> input hex / wedge
    // chunks (chunks.cu)
    int nchunk = 0, chunk_lmax = 0;
    std::vector<int> chunk_col_start;  // chunk colours
    int* d_ch_elem = nullptr;     // nchunk+1
    int* d_ch_node = nullptr;     // nchunk+1
    int* d_ch_nodes = nullptr;    // chunk-local -> global node
    int* d_ch_cstart = nullptr;   // slot-list offsets (+1)
    unsigned short* d_ch_csr = nullptr;
    ushort4* d_ch_lien = nullptr;
    // one 16-byte aligned record per chunk for the bulk copies of the pipelined linearized
    // product (chunk_record_words): header, node ids, connectivity, slot lists, slot offsets
    uint4* d_ch_rec = nullptr;
    int* d_ch_rec_off = nullptr;  // nchunk+1, in 16-byte units
    int chunk_rec_max = 0;        // largest record, bytes
    // the FP32 base state and coordinates packed per node (yb0..yb4, x0, x1, x2): two 16-byte
    // copies per node instead of eight 4-byte ones; rebuilt whenever d_yf is written
    float4* d_xbf = nullptr;
    int4* d_ienb = nullptr;       // Eb (face nodes first)
    int* d_iBCB = nullptr;        // Eb
    double* d_BCB = nullptr;      // Eb*18  [e][n][6]
    std::vector<int> perm_e;      // colour-sorted position -> input element id
    // host connectivity for the sparse solver's adjacency: tets in input order,
    // hexes and wedges in the colour order of d_ienh / d_ienw
    std::vector<int> h_ien, h_ienh, h_ienw;
    SparseCtx sp;

    double* d_x = nullptr;        // N*3
    float* d_xf = nullptr;        // N*3
    float* d_xlo = nullptr;       // N*3: x - (double)d_xf, rounded to float
    int* d_iBC = nullptr;         // N
    double* d_BC = nullptr;       // N*6  [n][6]
    float* d_BCf = nullptr;
    int* d_iper = nullptr;        // N
    int nmaster = 0;              // masters with slaves
    int* d_mst = nullptr;         // masters
    int* d_slv_start = nullptr;   // nmaster+1
    int* d_slv = nullptr;         // slaves (ascending)
    int nslave = 0;
    int* d_slaves = nullptr;      // all slave nodes
    int nbcn = 0;                 // nodes with a Dirichlet/flux bit
    int* d_bcn = nullptr;

    // state (FP64 master copies + FP32 shadows)
    double *d_y = nullptr, *d_ac = nullptr, *d_yold = nullptr, *d_acold = nullptr;
    float *d_yf = nullptr, *d_acf = nullptr;
    float* d_ylo = nullptr;       // y - (double)d_yf, rounded to float (double-float residual)
    double* d_qres = nullptr;     // idiff = 1: reconstructed diffusive flux, 13 per node (12 + lumped mass)
    float* d_qresf = nullptr;     //   its FP32 copy for the mixed outer residual
    // hex/wedge split residual: per (element, node, direction) I_a,i = sum_q W_q N_a,i as hi/lo
    bool split_ready = false;
    float2* d_Ih = nullptr;
    float2* d_Iw = nullptr;

    // work arrays
    double *d_res = nullptr, *d_rmes = nullptr, *d_bd = nullptr, *d_Dy = nullptr, *d_bdstage = nullptr;
    double *d_ypre = nullptr, *d_t64 = nullptr, *d_t64b = nullptr;
    float *d_resf = nullptr, *d_rmesf = nullptr, *d_bdf = nullptr, *d_t32 = nullptr, *d_t32b = nullptr;
    void* d_U = nullptr;          // Krylov basis (Kspace+1) x ldU, double or float
    size_t ldU = 0;               // 5N rounded up to 64 values: every basis vector starts on 256 bytes
    int Ucap = 0;
    double* d_scal = nullptr;     // device scalars (see Scal below)
    double* d_part = nullptr;     // reduction partials
    unsigned int* d_count = nullptr;
    int* d_flag = nullptr;        // [0] converged, [1] error bits, [2] Krylov iterations of the cycle
    CycleGraph cyc;
    CycleGraph cyc_net;           // the learned preconditioner's flexible GMRES cycle
    StepGraph stepg;              // the whole time step
    NetCtx net;
    int lin_pipe_grid = 1;        // its CTAs per colour launch (resident slots) of the chosen variant
    int ress_pipe_grid = 1;       // the same for the pipelined split outer residual
    // autotuned register/occupancy variants of the two pipelined sweeps (elements.cu): the
    // minimum CTAs per SM each is compiled for (linearized product 3 or 4, split residual 2, 3
    // or 4), their resident grids, the device time each took when tuned (ms, -1 untimed), and
    // whether they were chosen by timing (tuned) or forced (phgpu_set_tuning)
    int lin_minb = 4, ress_minb = 3;
    int lin_grids[2] = {1, 1}, ress_grids[3] = {1, 1, 1};
    double tune_ms[5] = {-1, -1, -1, -1, -1};
    bool tuned = false, tune_forced = false, tune_always = false;
    double* h_scal = nullptr;     // pinned mirror
    int* h_flag = nullptr;

    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool timing = true;
};

// device scalar slots (d_scal)
enum Scal : int {
    S_BETA = 0,        // running MGS beta
    S_UNORM = 1,
    S_EPSNRM = 2,
    S_ECHECK = 3,
    S_TMP0 = 4, S_TMP1 = 5, S_TMP2 = 6, S_TMP3 = 7,
    S_EB = 8,          // eBrg[K+1]
    S_RC = 8 + 64,     // Rcos[K]
    S_RS = 8 + 128,    // Rsin[K]
    S_YB = 8 + 192,    // yBrg[K]
    S_H = 8 + 256,     // H (K+1) x K, column-major
    S_TOTAL = 8 + 256 + 65 * 64
};
constexpr int kMaxK = 63;

template <typename R> Phys<R> make_phys(const phgpu_config& c);

// ---- element kernels (elements.cu) ----
enum ResMode : int { RM_RES = 1, RM_MODRES = 2, RM_LIN = 3 };
template <typename R>
void launch_elem_res(Ctx& C, int mode, const R* x, const R* ya, const R* yb, const R* ac,
                     R* out, int iabres, const int* skip, const R* ql = nullptr);
template <typename R>
void launch_elem_full(Ctx& C, const R* x, const R* y, const R* ac, R* res, R* rmes, R* bd, const R* ql = nullptr);
// idiff = 1: lumped L2 reconstruction of the diffusive flux (13 per node: 12 flux, 1 mass), then qpbc
template <typename R>
void launch_qrec(Ctx& C, const R* x, const R* y, R* out);
template <typename R>
void qpbc(Ctx& C, R* q13);
void launch_boundary(Ctx& C, const double* y, double* res);  // tets, then the hex and wedge blocks
int bnd_setup(Ctx& C, const phgpu_mesh* m);                    // boundary.cu
void bnd_free(Ctx& C);
void launch_bnd_blocks(Ctx& C, const double* y, double* res);
inline bool has_boundary(const Ctx& C) { return C.Eb > 0 || !C.bblk.empty(); }
void launch_elem_resh(Ctx& C, const double* y, const double* ac, const float* yf, const float* acf, double* out);
// outer residual with no FP64 arithmetic: double-float element-constant flux + FP32 increments
void launch_elem_ress(Ctx& C, const float* yh, const float* ylo, const float* acf, double* out,
                      const float* ql = nullptr);
// the same for the hex and wedge blocks (topo_ress.cu); topo_split_setup forms I_a,i once
int topo_split_setup(Ctx& C);
void launch_topo_ress(Ctx& C, const float* yh, const float* ylo, const float* acf, double* out, const float* ql);
// hex and wedge blocks; mode RM_RES/RM_MODRES/RM_LIN or 4 (ires = 3 + block diagonal)
template <typename R>
void launch_topo(Ctx& C, int mode, const R* x, const R* ya, const R* yb, const R* ac, R* res, R* rmes, R* bd,
                 int iabres, const int* skip, const R* ql = nullptr);
int upload_tables(Ctx& C);
int build_chunks(Ctx& C, const int* ien, const double* x_ref);
// 4-byte words of a chunk record of ne elements and nn nodes, and the word offsets of its parts:
// header {e0, ne, n0, nn}; node ids (nn); connectivity (ne ushort4); slot lists (4 ne ushort);
// slot-list offsets relative to the chunk's first slot (nn + 1) -- each part padded to 16 bytes
__host__ __device__ constexpr int rec_pad4(int w) { return (w + 3) & ~3; }
__host__ __device__ constexpr int rec_ids_off() { return 4; }
__host__ __device__ constexpr int rec_lien_off(int nn) { return 4 + rec_pad4(nn); }
__host__ __device__ constexpr int rec_csr_off(int ne, int nn) { return rec_lien_off(nn) + rec_pad4(2 * ne); }
__host__ __device__ constexpr int rec_cst_off(int ne, int nn) { return rec_csr_off(ne, nn) + rec_pad4(2 * ne); }
__host__ __device__ constexpr int chunk_record_words(int ne, int nn) { return rec_cst_off(ne, nn) + rec_pad4(nn + 1); }
// write the FP32 base state d_yf into the packed node records d_xbf (after every write of d_yf)
void pack_xb(Ctx& C);
// bit of flag[1] that the pipelined linearized product sets when a bulk copy did not complete
constexpr int kPipeCopyFailed = 8;
constexpr int kMbarTriesMax = 1 << 19;  // tries of a bounded mbarrier wait before it gives up (~2 s)
constexpr const char* kPipeCopyMsg = "pipelined linearized product: a bulk copy did not complete in time";
int configure_element_kernels(Ctx& C);
// time the variants of the pipelined linearized product and split residual on the resident
// FP32 state (d_yf, d_ylo, d_acf) and keep the fastest of each (no-op once tuned or forced)
int autotune_sweeps(Ctx& C);
void select_sweep_variants(Ctx& C, int lin_minb, int ress_minb);

// ---- nodal kernels (nodal.cu) ----
template <typename R> void bc3res(Ctx& C, R* r);
template <typename R> void bc3per(Ctx& C, R* r);
template <typename R> void bc3bdg(Ctx& C, const double* y, R* bd);
template <typename R> void itrbc_pert(Ctx& C, R* v, bool zero_dirichlet);
void itrbc_state(Ctx& C, double* y, double* ac, bool with_ac);
template <typename R> void lu_fact(Ctx& C, R* bd, int* flag);
// FP32 blocks bdf factored in FP64 into bd, and the factors rounded back into bdf (mixed precision)
void lu_fact_f32(Ctx& C, float* bdf, double* bd, int* flag);
template <typename R, typename V> void lu_apply(Ctx& C, const R* bd, V* r, int code);
template <typename R, typename V> void lu_apply(Ctx& C, const R* bd, const V* in, V* out, int code);
void ref_to_dev_state(Ctx& C, const double* h_ref, double* d_tmp_host_layout, double* d_out);
void dev_to_ref_state(Ctx& C, const double* d_in, double* d_tmp, double* h_ref);
void ref_to_dev_res(Ctx& C, const double* h_ref, double* d_tmp, double* d_out);
void dev_to_ref_res(Ctx& C, const double* d_in, double* d_tmp, double* h_ref);
void ref_to_dev_bd(Ctx& C, const double* h_ref, double* d_tmp, double* d_out);
void dev_to_ref_bd(Ctx& C, const double* d_in, double* d_tmp, double* h_ref);
void to_f32(Ctx& C, const double* a, float* b, size_t n);
// hi = (float)a, lo = (float)(a - hi): the double-float pair of each value
void split_f32(Ctx& C, const double* a, float* hi, float* lo, size_t n);
void to_f64(Ctx& C, const float* a, double* b, size_t n);
void fill0(Ctx& C, void* p, size_t bytes);

// reductions with FP64 accumulation into d_scal[slot] (deterministic)
template <typename V> void dot(Ctx& C, const V* a, const V* b, size_t n, int slot, const int* skip);
// MGS step: w -= d_scal[S_H + (jprev)]*uprev (if uprev), then H[...] = w.uj
template <typename V>
void mgs_step(Ctx& C, V* w, const V* uprev, const double* beta_prev, const V* uj, size_t n,
              double* beta_out, const int* skip);
template <typename V> void scale_by(Ctx& C, V* w, const double* s, int mode, size_t n, const int* skip);

// ---- sparse solver (sparse.cu, tangent.cu) ----
// genadj.f: the unique neighbours of every node over all element blocks, ascending (1-based)
void block_adjacency(int N, const int* ien, int ne, const int* ienh, int nh, const int* ienw, int nw,
                     std::vector<int>& colm, std::vector<int>& rowp);
int sparse_setup(Ctx& C);
int ebe_setup(Ctx& C);    // PHGPU_ERR_UNSUPPORTED unless the mesh has one element topology
// element tangents stored per element (ElmGMRe), bd += their diagonal blocks
template <typename R> void launch_tangent_ebe(Ctx& C, const R* x, const R* y, R* EG, R* bd);
template <typename R> void i3pre(Ctx& C, const R* bd, R* EG);
// Au1GMR + bc3per: q = sum_e EG_e p(iper)
template <typename M, typename V> void ebe_ap(Ctx& C, const M* EG, const V* p, V* q);
template <typename R> void launch_tangent(Ctx& C, const R* x, const R* y, R* lhsK, R* bd = nullptr);
int upload_tangent_tables(Ctx& C);
int configure_tangent_kernels(Ctx& C);
// Spsi3pre: lhsK <- L_i^-1 lhsK U_j^-1 with the i3LU factors bd (device layouts)
template <typename R> void spsi3pre(Ctx& C, const R* bd, R* lhsK);
// SparseAp + bc3per: q = lhsK p(iper), slaves summed into masters
template <typename M, typename V> void sparse_ap(Ctx& C, const M* lhsK, const V* p, V* q);
// greedy first-fit element colouring (solver.cu)
int colour(Ctx& C, int n_nodes, const int* ien, int nen, int ne, std::vector<int>& order, std::vector<int>& start);

// a named range on the NVTX timeline of a profiler (host-side phases; no cost without a tool)
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};
int check(Ctx& C, cudaError_t e, const char* what);
int fail(Ctx& C, int code, const std::string& msg);
// The dynamic shared memory a kernel may be launched with.  Function attributes belong to the
// process (per device), not to a context, so a context never lowers one to its own mesh's need
// (another context's launches would then fail): every call checks the need against the
// device's opt-in limit less the kernel's static shared memory and sets the attribute to that
// limit.  Occupancy follows the shared memory of each launch, not this attribute.
template <typename F>
inline cudaError_t smem_attr(F f, cudaFuncAttribute attr, int need) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, f);
    if (e != cudaSuccess) return e;
    const int limit = optin - (int)fa.sharedSizeBytes;
    if (need > limit) return cudaErrorInvalidValue;
    return cudaFuncSetAttribute(f, attr, limit);
}
// host <-> device copies and clears of a context, all on its own stream (ordered after the
// context's kernels; never the legacy stream, which neither orders against a non-blocking
// stream nor may synchronise while another thread captures a graph): the copies are complete
// on return, the clear is ordered before the context's next work
int h2d(Ctx& C, void* dst, const void* src, size_t bytes, const char* what);
int d2h(Ctx& C, void* dst, const void* src, size_t bytes, const char* what);
int dzero(Ctx& C, void* dst, size_t bytes, const char* what);

// ---- learned preconditioner (learn.cu) ----
int net_setup(Ctx& C);                      // graph, buffers and the Z basis (first use)
int net_prepare(Ctx& C);                    // context features of the current state and FP32 LU factors
void net_apply(Ctx& C, const float* v, float* z);   // z = P(v), four kernels, graph-capturable
void net_free(Ctx& C);
// training pair `slot`: v = Aw / ||Aw||, t = w / ||Aw|| (||Aw||^2 at nrm2 on the device), current features
int net_store_pair(Ctx& C, int slot, const float* Aw, const float* w, const double* nrm2);
bool net_usable(const Ctx& C);              // graph and weights present

}  // namespace phgpu

struct phgpu_ctx {
    phgpu::Ctx c;
};
