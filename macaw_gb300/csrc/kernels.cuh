// Descriptor types shared by the host planner (engine.cu) and the kernels (kernels.cu).
//
// Every batched kernel walks an array of descriptors; each descriptor carries its
// own pointers and shapes, so one launch can serve many terms, modes, states or
// ensemble members of different sizes (ragged batching).  A tensor is addressed
// the way the reference lays it out (init_calc.f90:531-536): for the mode being
// touched, element (l, j, r) sits at l + L*(j + n*r), with L = prod of the
// sizes of the faster modes and R = prod of the sizes of the slower modes.
#pragma once
#include <vector>
#include "common.cuh"

#define MAXDOF_MODE 4     // primitive DOFs combined in one DVR logical mode
#define HOLE_TILE 32      // fibres staged per shared-memory tile in hole_kernel
#define HOLE_THREADS 256

// Y = alpha * (M_eff x_mode X) (+ Y when accumulate)
// Tensor storage formats.  TF_C64: complex128 (re, im).  TF_SPLIT: the same 16
// bytes per element as FP32 (re hi, im hi, re lo, im lo), re = hi + lo to
// ~2^-48 relative: intermediates of the split-precision chains stay in this
// form, so neither side of a chain step converts through the FP64 pipe.
enum { TF_C64 = 0, TF_SPLIT = 1, TF_F32 = 2 };

struct ProdDesc {
  const cplx* X;
  cplx* Y;
  const cplx* M;           // column-major, leading dimension ldm
  long long L, R;
  int nin, nout, ldm;
  int conjT;               // 0: M_eff(j',j) = M[j' + ldm*j];  1: M_eff(j',j) = conj(M[j + ldm*j'])
  cplx alpha;
  int accumulate;
  int xfmt, yfmt;          // TF_*: TF_SPLIT output only with alpha = 1, no accumulation, PREC > 0
  int pad;
  long long block_start;
};

// Partial single-hole contraction C(j1,j2) = sum_{l,r} conj(X(l,j1,r)) Y(l,j2,r)
struct HoleDesc {
  const cplx* X;
  const cplx* Y;
  long long L, R;
  int n1, n2;
  cplx* partial;           // [nblk][n1*n2]
  long long block_start;
  int nblk;
  int xfmt, yfmt;          // TF_*
  int pad;
};

// out (n1 x n2, leading dim ld) = [out +] sum_t alpha_t * sum_blocks partial_t
struct RedTarget {
  cplx* out;
  int n1, n2, ld;
  int hermitize;           // out = 1/2 (S + S^H)
  int first, count;
  int accumulate;
  int pad;
};
struct RedTerm {
  const cplx* partial;
  int nblk;
  int conjT;               // 1: the term adds alpha * (its partials' matrix)^H (n2 x n1 source)
  cplx alpha;
};

// h1mode of one (mode, operator): apply the primitive DOF operators to the SPFs
// of the right state (hamilton.f90:447-471) and project on the left SPFs
// (zher2k / zgemm, hamilton.f90:475-482).
struct H1Desc {
  const cplx* phi_r;
  const cplx* phi_l;
  cplx* ophi;              // G x n2, operator applied to phi_r
  cplx* h;                 // n1 x n2 (ld n1); nullptr: only ophi is produced
  cplx* X;                 // n1 x n2 scratch: phi_l^H ophi before the Hermitian part
  int G, n1, n2;
  int same_state;
  int ndof;
  int ng[MAXDOF_MODE];
  int optype[MAXDOF_MODE]; // 0 none, 1 dense real, 2 diagonal, 3 dense imaginary (i x real)
  const cplx* mat[MAXDOF_MODE];
  const float2* matf[MAXDOF_MODE];  // the real coefficients split into FP32 (hi, lo)
};

// Regularised inverse of a Hermitian n x n matrix by Jacobi rotations
// (StdRegInv, maths.f90:8-83), then out_k = inv * mf_k for the listed operators.
struct RegInvDesc {
  const cplx* A;           // n x n (ld n), Hermitian
  cplx* inv_out;           // optional n x n copy of the regularised inverse
  int n;
  int regtype;             // 0 'poly', 1 'tikh'
  double eps;
  int op_first, op_count;
  // optional warm start: the eigenvectors of the previous call (n x n) and the
  // number of consecutive warm starts behind them (0: none yet)
  cplx* vprev;
  int* vcount;
};
struct MFOp {
  const cplx* mf;          // n x n2 (ld n)
  cplx* out;               // n x n2 (ld n)
  int n2;
  int pad;
};

// SPF derivative of one DVR mode and state (derivatives.f90:96-153):
// dphi = f * sum_k ophi_k * rhom1MF_k^T, then dphi -= phi (phi^H phi)^-1 phi^H dphi.
struct SpfDesc {
  const cplx* phi;         // G x n
  long long out_offset;    // offset of the block in the output vector
  int G, n;
  int op_first, op_count;
  cplx* partial;           // [ntile][2 n^2]: per grid tile phi^H phi and phi^H dphi
  cplx* X;                 // n x n: (phi^H phi)^-1 phi^H dphi
  long long block_start;   // first tile block of this descriptor
  int ntile;
  int pad;
};
#define SPF_TILE 32          // grid rows per block of the tiled SPF derivative
struct SpfOp {
  const cplx* ophi;        // G x n2
  const cplx* rm;          // n x n2 (ld n)
  int n2;
  int pad;
};

// Elementwise weighted sum of source tensors into a range of the output vector.
struct SumRange {
  long long offset, n;
  int first, count;
};
struct SumSrc {
  const cplx* src;
  cplx coeff;
  int fmt;                 // TF_*
  int pad;
  float cs[4];             // coeff split into FP32 pairs (re hi, re lo, im hi, im lo), set by split_coeffs
};
// Fill SumSrc::cs from coeff for the compensated term sums (host, before upload).
inline void split_coeffs(std::vector<SumSrc>& v) {
  for (auto& s : v) {
    const float rh = (float)s.coeff.x, ih = (float)s.coeff.y;
    s.cs[0] = rh;
    s.cs[1] = (float)(s.coeff.x - (double)rh);
    s.cs[2] = ih;
    s.cs[3] = (float)(s.coeff.y - (double)ih);
  }
}

// out (n1 x n2, ld n1) = sum_k coeff_k * src_k  (operators pre-summed per state and mode)
struct MatSumDesc {
  cplx* out;
  int n1, n2;
  int first, count;
};
struct MatSumSrc {
  const cplx* src;
  cplx coeff;
};

struct SpfErrDesc {
  const cplx* ds;          // n x n overlap of the SPF difference
  const cplx* rho;         // n x n density matrix (frozen)
  int n, mode;
};

struct NatpopDesc {       // one (mode, state) block of the natural populations (output.f90:88-140)
  const cplx* rho;         // n x n density matrix (upper triangle authoritative)
  const cplx* S;           // Gaussian modes: S00 of the set (n x n), else null
  cplx* work;              // Gaussian modes: 2 n^2 scratch
  double* natpop;          // n, decreasing
  double* ggp;             // Gaussian modes: gross Gaussian populations (n)
  double* poperr;          // Gaussian modes: population errors (n, decreasing)
  int n, pad;
};
void launch_natpop(const NatpopDesc* d, int nd, int* status, cudaStream_t st);

// Calc_Density (output.f90:332-445) of one state along one DOF
struct DensGridArgs {      // grid DOF: SPFs phi(ll, nG, nl, n) of the mode, DOF in the middle
  const cplx* phi;
  const cplx* rho;         // n x n (upper triangle authoritative)
  cplx* Y;                 // scratch G x n (rho applied to the SPFs)
  cplx* DM;                // scratch nG x nG (density matrix of the DOF)
  const double* trafo;     // basis x grid (ld ldt), or null
  double* dens;            // nG
  double* pop;             // nG (basis populations), with trafo
  int n, nG, ll, nl, ldt, pad;
};
struct DensGwpArgs {       // Gaussian DOF k of a mode with nmd DOFs
  const cplx* xi;          // parameters (nmd x n)
  const double* a;         // widths (lda x n)
  const cplx* rho;         // n x n
  double* dens;            // nG
  double x0, delta;
  int n, nmd, lda, k, nG, pad;
};
void launch_density_grid(const DensGridArgs& a, cudaStream_t st);
void launch_density_gwp(const DensGwpArgs& a, cudaStream_t st);

struct SnapSeg {
  cplx* ptr;               // matrix storage
  long long offset;        // first index in the flat snapshot
  int density;             // 1: a density matrix, 0: a mean field
  int pad;
};
// Learned mean-field extrapolation: five step-start snapshots, 20 network inputs
// (Newton increments of orders 1-4 at the half step and the step end, Re/Im, and
// four step-length ratios), 4 outputs (Re/Im residual at the half step and end).
#define MFX_NHIST 5
#define MFX_NFEAT 20
#define MFX_NOUT 4
struct MfxHist {
  const cplx* z[MFX_NHIST];  // oldest first
};
struct MfxCoef {
  double inc[2][MFX_NHIST - 1][MFX_NHIST];  // [half, end][order-1][history point]
  double base[2][MFX_NHIST];                // quartic extrapolation weights (all five points)
  double ratio[MFX_NHIST - 1];              // (t1-t0, t2-t1, t3-t2, h) / (t4-t3)
  double fscale[MFX_NFEAT];                 // input column scales
  double tscale[MFX_NOUT];                  // output column scales
};

struct StageArgs {
  const cplx* k[7];
  double c[7];
  int nk;
};

// Launch helpers (kernels.cu)
bool tc_enabled();
void tc_prepare();
bool launch_prod_tc(const ProdDesc* d_descs, int ndesc, long long nblocks, int maxn, cudaStream_t st, bool force);
int tc_timeout_flag(bool clear);
// persist > 0: at most `persist` persistent CTAs walk the batch's blocks
void launch_prod(const ProdDesc* d_descs, int ndesc, long long nblocks, int maxn, cudaStream_t st,
                 int prec = 0, int tc = 1, int persist = 0);
void launch_hole(const HoleDesc* d_descs, int ndesc, long long nblocks, cudaStream_t st, int prec = 0,
                 int persist = 0);
void launch_reduce(const RedTarget* d_tg, int ntg, const RedTerm* d_terms, cudaStream_t st);
// with_h: also h1mode (second launch: the Hermitian part of same-state matrices);
// prec > 0: the operator products and phi^H (O phi) in compensated split FP32
void launch_h1(const H1Desc* d_descs, int ndesc, int maxn2, size_t smem_bytes, bool with_h, cudaStream_t st,
               int prec);
void launch_reginv(const RegInvDesc* d_descs, int ndesc, const MFOp* d_ops, int* d_status, cudaStream_t st);
// prec > 0: the tile products in compensated split FP32 (spf_tile_split_kernel)
// nf: the largest SPF count of the descriptors and their operators (<= 16: the
// two-group split tile kernel)
void launch_spf(const SpfDesc* d_descs, int ndesc, long long ntiles, const SpfOp* d_ops, cplx* out,
                cplx der_factor, int* d_status, cudaStream_t st, int prec, int nf = 0);
// prec > 0: compensated split-FP32 accumulation (termsum_split_kernel)
// A sum over a whole launch fused into a streaming kernel: v the vector to dot
// with (termsum: <v|out>; Lanczos axpy: any non-null v requests ||Kn||^2), partial
// one complex per block of the launch, counter zero-initialised, result in res.
#define FUSED_BLOCKS 608   // grid of the streaming kernels that carry a fused sum (4 per SM)
struct FusedDot {
  const cplx* v;
  cplx* partial;
  unsigned* counter;
  cplx* res;
};
// ---------------------------------------------------------------------------
// Statistical mixtures and dissipation (gmctdh_objects.f90:481-1141,
// derivatives.f90:70-83, 238-242).  The coefficients of every state are stored
// packet-minor: state s occupies [off, off + P n) with packet W at off + W n.
// ---------------------------------------------------------------------------
#define MAX_PACKETS 16
#define MAX_DISS1 4
#define PK_GRAM_BLOCKS 32   // one warp lane per block sum in pk_coef_kernel
struct PkState {
  long long off, n;        // storage offset of the state's block, configurations per packet
};
// <X_i | Y_j> summed over the states
struct PkGramPair {
  const cplx* X;
  const cplx* Y;
  int i, j;
};
// Pair order: (has2) P^2 pairs <A_i | (sum_t f ae_t W_t) A_j> at i + P j; then per
// type-1 operator k the P^2 pairs <A_i | V_k A_j> (plain coefficient dots, as the
// reference's zdotu / zgemm).  The packet norms WPpop = norm_wf(A_W) carry the SPF
// overlaps and come from an overlap plan (norms[3 W]).
struct PkCoefArgs {
  int P, ndiss1, has2, npairs;
  double eps_pop;
  double aeD1[MAX_DISS1];
  const cplx* partial;     // [npairs][PK_GRAM_BLOCKS]
  const cplx* norms;       // [3 P]: <A_W|A_W> with the SPF metric at 3 W
  double* pop;             // [P] WPpop (1 for a single packet)
  cplx* C1;                // [ndiss1][P][P]: D_W += sum_j (V_k A)_j C1[j + P W]
  cplx* C2;                // [ndiss1][P][P]: AuxA_k,W = sum_j A_j C2[j + P W]
  cplx* ML;                // [P][P]: dA_W += sum_j A_j ML[j + P W]  (multLagDiag I + i multLag)
};
// out[s][W] (+)= sum_j in[s][j] C[j + P W] for every state s and packet W (out0, if
// not null, replaces every descriptor's out)
struct PkMix {
  const cplx* in;
  const cplx* C;
  cplx* out;
  int accumulate;
};
void launch_pk_gram(const PkGramPair* d_pairs, int npairs, const PkState* d_st, int nstates, cplx* partial,
                    cudaStream_t st);
void launch_pk_coef(const PkCoefArgs& a, cudaStream_t st);
void launch_pk_mix(const PkMix* d_mix, int nmix, const PkState* d_st, int nstates, long long n1tot, int P,
                   cplx* out0, cudaStream_t st);

void launch_termsum(cplx* out, const SumRange* d_ranges, int nranges, const SumSrc* d_srcs,
                    long long total, cudaStream_t st, int prec,
                    FusedDot dot = FusedDot{nullptr, nullptr, nullptr, nullptr});
void launch_stage(cplx* out, const cplx* base, const StageArgs& a, double dt, long long n, cudaStream_t st);
// Bulirsch-Stoer: the last modified-midpoint stage 0.5 (am + an + dt d) (mmid,
// integrator.f90:550-551) and one polynomial-extrapolation column (pzextr, :559-608)
struct BsExtr {
  cplx* q[10];             // qA(:, 1..iEst) (index 0 unused)
  double f1[10], f2[10];   // per k1 = 1..iEst-1
  int iest;
  int pad;
};
void launch_bs_final(cplx* out, const cplx* am, const cplx* an, const cplx* d, double dt, long long n, cudaStream_t st);
void launch_bs_extr(const BsExtr& e, const cplx* est, cplx* a0, cplx* a1, long long n, cudaStream_t st);
// ensembles: member m owns elements off[m] .. off[m+1] of the vectors
void launch_ens_stage(cplx* out, const cplx* base, const StageArgs& a, const double* dt, const long long* off, int nm,
                      long long n, cudaStream_t st);
void launch_ens_accept(cplx* y, const cplx* src, const int* accept, const long long* off, int nm, long long n,
                       cudaStream_t st);
void launch_copy_scale(cplx* out, const cplx* in, cplx s, long long n, cudaStream_t st);
void launch_axpy(cplx* y, const cplx* x, cplx a, long long n, cudaStream_t st);
// out (complex FP32, TF_F32 storage) = in rounded to nearest
void launch_to_f32(cplx* out, const cplx* in, long long n, cudaStream_t st);
void launch_to_split(cplx* out, const cplx* in, long long n, cudaStream_t st);
void launch_gemv_cols(cplx* out, const cplx* basis, long long ld, const cplx* coef, int ncol, long long n,
                      cudaStream_t st);
void launch_jacobi_tridiag(const double* alpha, const double* beta, int n, double* evals, double* evecs,
                           int* d_status, cudaStream_t st);
void launch_matsum(const MatSumDesc* d_descs, int ndesc, const MatSumSrc* d_srcs, cudaStream_t st);
void launch_stage_modes(cplx* out, const cplx* base, const StageArgs& a, const double* dt_mode,
                        const unsigned char* elem_mode, long long off, long long n, cudaStream_t st);
void launch_masked_copy(cplx* y, const cplx* src, const unsigned char* elem_mode, const int* accept, long long off,
                        long long n, cudaStream_t st);
void launch_spf_err(const SpfErrDesc* d, int nd, double* err_mode, int nmodes, cudaStream_t st);
void launch_lan_axpy(cplx* Kn, const cplx* Kj, const cplx* Kp, const cplx* dot_alpha, const double* beta_prev,
                     double* alpha_out, long long n, cudaStream_t st,
                     FusedDot nrm = FusedDot{nullptr, nullptr, nullptr, nullptr});
void launch_lan_normalize(cplx* out, const cplx* in, const cplx* nrm2, double* beta_out, long long n, cudaStream_t st,
                          cplx* copy = nullptr, cplx* f32 = nullptr);
// <a|b> = sum_i conj(a_i) b_i in FP64 into *out, one launch, fixed summation order.
// partial: DOT_BLOCKS complex scratch; counter: one zero-initialised unsigned.
#define DOT_BLOCKS 304
void launch_dot(const cplx* a, const cplx* b, long long n, cplx* partial, unsigned* counter, cplx* out,
                cudaStream_t st);
void launch_snap(const SnapSeg* segs, int nseg, cplx* flat, long long E, int scatter, cudaStream_t st);
void launch_mfx_features(const MfxHist& hz, const MfxCoef& c, double* S, float* X, long long E, cudaStream_t st);
void launch_mfx_combine(const MfxHist& hz, const MfxCoef& c, const float* Y, const double* S, cplx* half, cplx* full,
                        long long E, cudaStream_t st);
// MLP forward on a given stream (mlp.cu): input buffer for M rows, then the output
struct mctdh_mlp;
float* mlp_input_buffer(mctdh_mlp* m, long long M);
const float* mlp_forward_on(mctdh_mlp* m, long long M, cudaStream_t st);
bool mlp_has_shape(const mctdh_mlp* m, int din, int dout);
double measure_fp64_tflops();

// ---------------------------------------------------------------------------
// Gaussian (G-MCTDH) modes (gwp.cu).  A Gaussian SPF j of a mode with d DOFs is
// g_j(x) = exp(sum_k a[k,j] x_k^2 + xi[k,j] x_k): widths a (real, fixed, GWPa
// layout a[k + lda*j]) and complex parameters xi (the psi block, xi[k + d*j]).
// ---------------------------------------------------------------------------
#define GWP_MAXDOF 16    // DOFs of one Gaussian mode
#define GWP_QR_PW 8      // panel width of the regularised least-squares QR

struct GwpOvlDesc {      // S(j1, j2) = <g1_j1 | g2_j2> (normalised), n1 x n2 (ld n1)
  const cplx* xi1;
  const cplx* xi2;
  const double* a;
  cplx* out;
  int nmd, lda, n1, n2;
  int kind;              // 0: same parameter set (diagonal 1, lower = conj upper); 1: full;
                         // 2: conjugate transpose of the full overlap with the sets swapped;
                         // 3: overlap of the difference of two parameter sets xi1 - xi2 (upper
                         //    triangle, Calc_Err_SPF, cmf2_derivatives.f90:294-315)
  int pad;
};
struct GwpH1Desc {       // h1mode of a Gaussian mode (hamilton.f90:494-524)
  const cplx* xi1;
  const cplx* xi2;
  const double* a;
  const cplx* S;         // overlap of the two parameter sets, n1 x n2
  cplx* out;
  int nmd, lda, n1, n2;
  int same_state;        // 1: Hermitian from the upper triangle
  int ops[GWP_MAXDOF];   // primitive operator code per DOF (0 = identity)
};
struct GwpYOp {          // one operator of the Y vector of Calc_CY (gmctdh_objects.f90:1285-1326)
  const cplx* xi2;       // parameters of the right state
  const cplx* S12;       // overlap (left state, right state), n x n2
  const cplx* h;         // h1mode of the operator, n x n2
  const cplx* mf;        // mean field of the operator, n x n2
  int n2;
  int ops[GWP_MAXDOF];
};
struct GwpCYDesc {       // one (Gaussian mode, state) block of Calc_CY and the parameter solve
  const cplx* xi;        // parameters (d x n)
  const double* a;
  const cplx* S;         // S00 (n x n)
  const cplx* Sm1;       // Tikhonov inverse of S00 (n x n)
  const cplx* rho;       // density matrix of the mode (n x n)
  cplx* Sa0;             // nG x n, nG = d * n
  cplx* Sa0Sm1;          // nG x n
  cplx* M;               // (2 nG) x (nG + 1) least-squares system [C, Y; eps I, 0], column-major
  cplx* R;               // nG x nG: R factor entries of the panels
  cplx* x;               // nG solution (parameter derivative before der_factor)
  long long dxi_offset;  // where der_factor * x goes in the derivative vector
  cplx* tau;             // n x n (derivatives.f90:201-234)
  int nmd, lda, n, nG;
  int op_first, op_count;
  double eps;            // eps_C
};
void launch_gwp_ovl(const GwpOvlDesc* d, int nd, cudaStream_t st);
// Tikhonov inverses (regtype 'tikh') of n <= 32 Hermitian matrices into inv_out, by QR
void launch_tikh_inv(const RegInvDesc* d, int nd, cudaStream_t st);
void launch_gwp_h1(const GwpH1Desc* d, int nd, cudaStream_t st);
// Calc_CY and the Tikhonov parameter solve (StdRegSol 'tikh', maths.f90:87-162)
// for nd (mode, state) blocks; maxG = max nG.  Then dxi = der * x and tau.
// part: scratch of nd * maxG * maxn * maxops complex (the terms of Y)
void launch_gwp_cy(const GwpCYDesc* d, int nd, int maxG, int maxn, int maxops, const GwpYOp* ops, cplx* part,
                   cudaStream_t st);
void launch_gwp_solve(const GwpCYDesc* d, int nd, int maxG, cplx der, cplx* out, int* status, cudaStream_t st);

// CMF2 with Gaussian modes (cmf2_base.f90, cmf2_derivatives.f90)
struct GwpIsqrtDesc {    // D = U^-1 with S = U^H U (InverseSquareRootU, maths.f90:621-644), DhS = D^H S
  const cplx* S;         // n x n, upper triangle authoritative
  cplx* D;
  cplx* DhS;
  int n, pad;
};
struct GwpDhdDesc {      // D1^H h D2 for one operator of a Gaussian mode (Calc_DHD, hamilton.f90:535-574)
  const cplx* h;         // n1 x n2 (full)
  const cplx* D1;        // n1 x n1
  const cplx* D2;        // n2 x n2
  cplx* out;             // n1 x n2 (full; Hermitian when same_state)
  int n1, n2, same_state, pad;
};
struct GwpDDerivDesc {   // dD = -tau D for one (Gaussian mode, set) block (cmf2_derivatives.f90:228)
  const cplx* tau;
  long long off;         // offset of the block in the D vectors
  int n, pad;
};
void launch_gwp_isqrt(const GwpIsqrtDesc* d, int nd, int* status, cudaStream_t st);
void launch_gwp_dhd(const GwpDhdDesc* d, int nd, cudaStream_t st);
void launch_gwp_dderiv(const GwpDDerivDesc* d, int nd, const cplx* Din, cplx* Dout, cudaStream_t st);
