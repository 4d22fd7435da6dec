// Descriptor types shared by the host planner (engine.cu) and the kernels (kernels.cu).
//
// Every batched kernel walks an array of descriptors; each descriptor carries its
// own pointers and shapes, so one launch can serve many terms, modes, states or
// ensemble members of different sizes (ragged batching).  A tensor is addressed
// the way the reference lays it out (init_calc.f90:531-536): for the mode being
// touched, element (l, j, r) sits at l + L*(j + n*r), with L = prod of the
// sizes of the faster modes and R = prod of the sizes of the slower modes.
#pragma once
#include "common.cuh"

#define MAXDOF_MODE 4     // primitive DOFs combined in one DVR logical mode
#define HOLE_TILE 32      // fibres staged per shared-memory tile in hole_kernel
#define HOLE_THREADS 256

// Y = alpha * (M_eff x_mode X) (+ Y when accumulate)
struct ProdDesc {
  const cplx* X;
  cplx* Y;
  const cplx* M;           // column-major, leading dimension ldm
  long long L, R;
  int nin, nout, ldm;
  int conjT;               // 0: M_eff(j',j) = M[j' + ldm*j];  1: M_eff(j',j) = conj(M[j + ldm*j'])
  cplx alpha;
  int accumulate;
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
  int pad;
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
  int G, n1, n2;
  int same_state;
  int ndof;
  int ng[MAXDOF_MODE];
  int optype[MAXDOF_MODE]; // 0 none, 1 dense (from the right), 2 diagonal
  const cplx* mat[MAXDOF_MODE];
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
};

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

struct SnapSeg {
  cplx* ptr;               // matrix storage
  long long offset;        // first index in the flat snapshot
};
struct MfxWeights {
  double h[3], f[3];       // Lagrange weights of t0, t1, t2 at the half step and the step end
};

struct StageArgs {
  const cplx* k[7];
  double c[7];
  int nk;
};

// Launch helpers (kernels.cu)
void launch_prod(const ProdDesc* d_descs, int ndesc, long long nblocks, int maxn, cudaStream_t st,
                 int prec = 0);
void launch_hole(const HoleDesc* d_descs, int ndesc, long long nblocks, cudaStream_t st, int prec = 0);
void launch_reduce(const RedTarget* d_tg, int ntg, const RedTerm* d_terms, cudaStream_t st);
void launch_h1(const H1Desc* d_descs, int ndesc, size_t smem_bytes, cudaStream_t st);
void launch_reginv(const RegInvDesc* d_descs, int ndesc, const MFOp* d_ops, int* d_status, cudaStream_t st);
void launch_spf(const SpfDesc* d_descs, int ndesc, long long ntiles, const SpfOp* d_ops, cplx* out,
                cplx der_factor, int* d_status, cudaStream_t st);
void launch_termsum(cplx* out, const SumRange* d_ranges, int nranges, const SumSrc* d_srcs,
                    long long total, cudaStream_t st);
void launch_stage(cplx* out, const cplx* base, const StageArgs& a, double dt, long long n, cudaStream_t st);
void launch_copy_scale(cplx* out, const cplx* in, cplx s, long long n, cudaStream_t st);
void launch_axpy(cplx* y, const cplx* x, cplx a, long long n, cudaStream_t st);
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
                     double* alpha_out, long long n, cudaStream_t st);
void launch_lan_normalize(cplx* out, const cplx* in, const cplx* nrm2, double* beta_out, long long n, cudaStream_t st);
void launch_snap(const SnapSeg* segs, int nseg, cplx* flat, long long E, int scatter, cudaStream_t st);
void launch_mfx_features(const cplx* z0, const cplx* z1, const cplx* z2, float r1, float r2, float* X, long long E,
                         cudaStream_t st);
void launch_mfx_combine(const cplx* z0, const cplx* z1, const cplx* z2, const MfxWeights& w, const float* Y,
                        double tscale, cplx* half, cplx* full, long long E, cudaStream_t st);
// MLP forward on a given stream (mlp.cu): input buffer for M rows, then the output
struct mctdh_mlp;
float* mlp_input_buffer(mctdh_mlp* m, long long M);
const float* mlp_forward_on(mctdh_mlp* m, long long M, cudaStream_t st);
double measure_fp64_tflops();
