/*
 * olcao_gpu.h -- C ABI of the GB300 implementation of OLCAO's per-SCF-iteration
 * hot path: Gaussian two/three-centre integrals, their Bloch sums into
 * H(k)/S(k), the valence-core orthogonalisation, the upper-packed integral
 * layout, Hamiltonian assembly and the per-k complex Hermitian generalised
 * eigen-solve.
 *
 * Every entry point takes plain pointers and sizes.  Arrays are column-major
 * (Fortran order) and complex numbers are interleaved (re, im) binary64, so a
 * Fortran caller passes its own arrays through ISO_C_BINDING unchanged.
 * Host pointers are copied in; "device" pointers must live on the context's
 * device.  Status 0 means success; any other value is an olc_status_t and
 * olc_last_error() returns the message.
 *
 * Reference interfaces replaced (paths within UMKC-CPG/olcao):
 *   olc_create                 setupSCF set-up: initializeLattice,
 *                              initializeFindVec, computePhaseFactors,
 *                              renormalizeBasis, makeAlpha*Dist
 *                              (src/olcao/OLCAO_Setup.f90:88-126,
 *                               src/olcao/lattice.f90:300-432,
 *                               src/olcao/kpoints.f90:286-310,
 *                               src/olcao/basis.f90:55-243,
 *                               src/olcao/gaussRelations.f90:64-278)
 *   olc_gauss_overlap          gaussOverlapOL / KE / MV / NP / EP (+ saveCurrentPair)
 *                              (src/olcao/integrals.F90:81-486, 490-900,
 *                               904-1320, 1324-1715, 1719-2122;
 *                               src/olcao/intgSaving.F90:56-550)
 *   olc_ortho_pack             orthoOL / ortho(opCode) + makeValeVale packing
 *                              (src/olcao/integrals.F90:2601-2853,
 *                               src/olcao/intgOrtho.F90:23-187)
 *   olc_assemble_hamiltonian   readPackedMatrix(Accum) + unpackMatrix
 *                              (src/olcao/secularEqn.F90:128-166,
 *                               src/olcao/matrixSubs.F90:248-355)
 *   olc_solve_zhegv            solveZHEGV (src/olcao/interfaces.F90:73-120)
 *   olc_scf_iteration          one pass of secularEqnAllKP with the
 *                              potential-dependent integrals recomputed
 *                              (src/olcao/secularEqn.F90:33-287,
 *                               src/uolcao/integrals.F90:2860-3605 fused form)
 *   olc_populate_states        populateStates: occupations and Fermi level
 *                              (src/olcao/populate.F90:132-578)
 *   olc_make_valence_rho       makeValenceRho: density and operator traces
 *                              (src/olcao/valeCharge.F90:34-420)
 */
#ifndef OLCAO_GPU_H
#define OLCAO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OLC_MAX_ALPHAS      32   /* atomic Gaussian exponents per atom type  */
#define OLC_MAX_RADIAL      12   /* radial functions per atom type           */
#define OLC_MAX_POT_ALPHAS  32   /* potential Gaussian exponents per type    */
#define OLC_MAX_STATES      40   /* basis states (l,m) per atom type         */

typedef enum {
  OLC_OK = 0,
  OLC_ERR_ARG = 1,            /* invalid argument / inconsistent sizes       */
  OLC_ERR_CUDA = 2,           /* CUDA runtime or library failure             */
  OLC_ERR_LATTICE = 3,        /* "More lattice points needed" (integrals.F90:249-255) */
  OLC_ERR_NOT_PD = 4,         /* S(k) not positive definite: ZHEGV info > n   */
  OLC_ERR_EIGEN = 5,          /* eigen-solver failed to converge: 0 < info <= n */
  OLC_ERR_ALLOC = 6,          /* device allocation failed                    */
  OLC_ERR_UNSUPPORTED = 7     /* feature outside this build (e.g. l > 3)     */
} olc_status_t;

/* One atom type (reference: atomTypes(i), src/olcao/atomicTypes.f90:40-120).
 * Radial functions are listed valence first, then core; coefficient arrays
 * hold numOrbAlphas(l+1) leading entries, the rest must be zero. */
typedef struct {
  int32_t element;                        /* element id, 1-based              */
  int32_t num_orb_alphas[4];              /* numOrbAlphas(1..4): s >= p >= d >= f */
  double  alphas[OLC_MAX_ALPHAS];         /* ascending                         */
  int32_t num_vale_radial;
  int32_t num_core_radial;
  int32_t radial_l[OLC_MAX_RADIAL];
  double  radial_coeff[OLC_MAX_RADIAL][OLC_MAX_ALPHAS];
} olc_atom_type_t;

/* One potential type (reference: potTypes(i), src/olcao/potTypes.f90:20-75). */
typedef struct {
  int32_t element;
  int32_t num_alphas;
  double  nuc_charge;                     /* Z, the nuclear factor            */
  double  nuc_alpha;                      /* Gaussian nuclear exponent        */
  double  alphas[OLC_MAX_POT_ALPHAS];     /* ascending                         */
} olc_pot_type_t;

/* Whole-system description.  All positions and vectors are in bohr.
 * real_vectors is realVectors(xyz, abc) column-major (column = a, b, c).
 * Potential sites of one type must be consecutive (the reference's
 * currPotNumber..+multiplicity-1 convention, integrals.F90:2527-2530). */
typedef struct {
  double real_vectors[9];
  int32_t num_atom_types;
  const olc_atom_type_t* atom_types;
  int32_t num_atom_sites;
  const int32_t* site_type;               /* [num_atom_sites], 0-based        */
  const double*  site_pos;                /* [3*num_atom_sites]               */
  int32_t num_pot_types;
  const olc_pot_type_t* pot_types;
  int32_t num_pot_sites;
  const int32_t* pot_site_type;           /* [num_pot_sites], 0-based         */
  const double*  pot_site_pos;            /* [3*num_pot_sites]                */
  int32_t num_kpoints;
  const double*  kpoints_abc;             /* [3*num_kpoints] fractional       */
  double basis_fn_thresh;                 /* BASIS_FN convergence, e.g. 1e-16 */
  int32_t rel;                            /* 1: scalar-relativistic, the mass-
                                             velocity term joins H (the
                                             reference's rel, OLCAO_Setup.f90:
                                             142-144); 0: non-relativistic  */
} olc_system_t;

/* Integral operators (the reference's opCode values, integrals.F90:2710-2853). */
typedef enum {
  OLC_OP_OVERLAP = 1,     /* gaussOverlapOL -> atomOverlap                    */
  OLC_OP_KINETIC = 2,     /* gaussOverlapKE -> atomKEOverlap                  */
  OLC_OP_NUCLEAR = 3,     /* gaussOverlapNP -> atomNucOverlap                 */
  OLC_OP_ELECPOT = 4,     /* gaussOverlapEP -> atomPotOverlap(term)           */
  OLC_OP_MASSVEL = 5,     /* gaussOverlapMV -> atomMVOverlap (with the driver's
                             minus sign, integrals.F90:1222-1236)            */
  OLC_OP_HAMILTONIAN = 6  /* KE + NP (+ MV) + sum_j c_j V_j in one pass (fused form) */
} olc_op_t;

typedef enum {
  OLC_PREC_FP64 = 0,      /* plain FP64 path                                  */
  OLC_PREC_MIXED = 1      /* eigen-solve in FP32 refined by error-free split-BF16
                             Rayleigh-Ritz products to FP64-grade eigenvalues;
                             integrals and assembly stay FP64                 */
} olc_precision_t;

typedef struct olc_context olc_context_t;

/* Sizes derived by olc_create (valeDim, coreDim, potDim, numKPoints, ...). */
typedef struct {
  int32_t vale_dim;
  int32_t core_dim;
  int32_t pot_dim;
  int32_t num_kpoints;
  int32_t num_cells;          /* numCellsReal                                 */
  int32_t num_pair_tasks;     /* surviving (atom pair, lattice cell) blocks    */
  int64_t packed_len;         /* vale_dim*(vale_dim+1)/2                       */
} olc_dims_t;

/* Library version and last error of the calling thread. */
const char* olc_version(void);
int olc_last_error(char* buf, size_t len);

/* Set-up: copies the system to the device and builds the lattice, k-point
 * phases, basis and screening tables.  stream may be NULL (legacy stream) or
 * a cudaStream_t the caller owns; all work of this context runs on it. */
int olc_create(const olc_system_t* sys, void* stream, olc_context_t** ctx);
int olc_destroy(olc_context_t* ctx);
int olc_get_dims(const olc_context_t* ctx, olc_dims_t* dims);
int olc_set_stream(olc_context_t* ctx, void* stream);

/* One integral pass for operator op (term = potential term index for
 * OLC_OP_ELECPOT, 0-based; coeffs[pot_dim] for OLC_OP_HAMILTONIAN, else NULL).
 * Writes the un-orthogonalised blocks saveCurrentPair produces, for all k:
 *   vv[vale_dim, vale_dim, nk] (upper triangle meaningful),
 *   cv[core_dim, vale_dim, nk], cc[core_dim, core_dim, nk]
 * as DEVICE complex128 arrays (any of cv/cc may be NULL when core_dim == 0). */
int olc_gauss_overlap(olc_context_t* ctx, int op, int term,
                      const double* coeffs, int precision,
                      double* vv, double* cv, double* cc);

/* Orthogonalise and pack, for all k (DEVICE arrays).  For the overlap
 * operator pass cv == s_cv.  Outputs packed[2, packed_len, nk] with the
 * reference's |x| < 1e-10 flush when core_dim > 0. vv is overwritten. */
int olc_ortho_pack(olc_context_t* ctx, int is_overlap, double* vv,
                   const double* cv, const double* cc, const double* s_cv,
                   double* packed);

/* H(k) packed = NP + KE (+ MV) + sum_j c_j V_j with the reference's rule
 * that a zero coefficient adds the term with factor 1 (matrixSubs.F90:
 * 278-282).  terms[nterm] are DEVICE pointers to packed[2, packed_len, nk]
 * arrays, coeffs[nterm] their multipliers. */
int olc_assemble_hamiltonian(olc_context_t* ctx, const double* const* terms,
                             const double* coeffs, int nterm, double* packed_h);

/* Generalised eigen-problem for every k: A x = lambda B x with A, B given
 * upper-packed (DEVICE).  Writes eigenvalues[num_states, nk] (Hartree,
 * ascending) and, if vectors != NULL, vectors[vale_dim, num_states, nk]
 * complex128.  info[nk] receives LAPACK-style info codes (host memory). */
int olc_solve_zhegv(olc_context_t* ctx, const double* packed_h,
                    const double* packed_s, int num_states,
                    double* eigenvalues, double* vectors, int32_t* info);

/* How the potential-dependent part of H(k) is produced each iteration. */
typedef enum {
  OLC_FORM_FUSED = 0,     /* V = sum_j c_j V_j recomputed from the integrals  */
  OLC_FORM_STORED = 1     /* V_j kept resident in HBM (OLCAOsetup's stored
                             integrals) and summed with the coefficients     */
} olc_form_t;

/* Flags of olc_scf_iteration. */
#define OLC_ITER_EIG_DEVICE   1   /* eigenvalues pointer is device memory    */
#define OLC_ITER_COEFF_DEVICE 2   /* coeffs pointer is device memory         */
#define OLC_ITER_GRAPH        4   /* mixed stored-form pass as a CUDA graph:
                                     the first call for a num_states / vectors
                                     choice runs directly, the second captures,
                                     later calls replay (direct launches if the
                                     capture is refused)                      */

/* Set-up of the iteration-invariant parts of the SCF pass: S(k) orthogonalised,
 * H0 = ortho(KE + NP (+ MV when rel = 1)), and for OLC_FORM_STORED every
 * orthogonalised, packed operator (NP, KE, MV when rel = 1, V_j) kept apart.
 * Must precede olc_scf_iteration. */
int olc_scf_prepare(olc_context_t* ctx, int precision, int form);

/* One SCF-iteration pass of the hot path (secularEqnAllKP): H(k) built with
 * the coefficients coeffs[pot_dim] in the prepared form, then the generalised
 * eigen-problem solved for all k.  eigenvalues[num_states, nk]; vectors
 * (DEVICE, may be NULL) as for olc_solve_zhegv; flags: OLC_ITER_*. */
int olc_scf_iteration(olc_context_t* ctx, const double* coeffs, int precision,
                      int num_states, double* eigenvalues, int flags,
                      double* vectors);

/* H(k) and S(k) as the prepared SCF pass builds them, for one k-point, as
 * full Hermitian complex128 [vale_dim, vale_dim] matrices (host or device
 * destination): lets a caller hand the secular equation to another solver
 * or write it out.  coeffs is a HOST array [pot_dim]. */
int olc_scf_matrices(olc_context_t* ctx, const double* coeffs, int kpoint,
                     double* h, double* s, int on_device);

/* FP64-accurate complex product C = A B (DEVICE, column-major, m x k times
 * k x n) formed error-free from BF16 slices on the tensor cores -- the product
 * the mixed-precision solver (OLC_PREC_MIXED) builds its Rayleigh-Ritz
 * matrices with.  Exposed for checking and for callers' own products. */
int olc_split_zgemm(olc_context_t* ctx, int m, int n, int k, const double* a,
                    const double* b, double* c);

/* FP32-accurate complex product C = op(A) B (DEVICE complex64, column-major;
 * op(A) = A (m x k, ld m) or, with conj_a, A^H of a k x m array (ld k)) from
 * three BF16 pieces per operand on the tensor cores -- the product the
 * mixed solver's FP32 stage uses for its reduction, back-transform and
 * Loewdin steps.  No reference counterpart (the reference's products are
 * LAPACK's FP64 BLAS); exposed for checking. */
int olc_split_cgemm32(olc_context_t* ctx, int m, int n, int k, const float* a, int conj_a,
                      const float* b, float* c);

/* Stage timing (CUDA events on the context's stream) and kernel counting.
 * Stages: the integral primitives, the basis contraction, the Bloch sum and
 * scatter, the orthogonalisation (GEMMs + pack), Hamiltonian assembly, and
 * the eigen-solve.  olc_profile_read synchronises the stream. */
typedef enum {
  OLC_STAGE_PRIMITIVES = 0,
  OLC_STAGE_CONTRACT = 1,
  OLC_STAGE_BLOCH = 2,
  OLC_STAGE_ORTHO = 3,
  OLC_STAGE_ASSEMBLE = 4,
  OLC_STAGE_SOLVE = 5,
  OLC_STAGE_REFINE = 6,        /* mixed precision: Loewdin step + cluster solves */
  OLC_STAGE_DENSITY = 7,       /* valence density and its traces               */
  OLC_STAGE_TRIDIAG = 8,       /* mixed precision: FP32 tridiagonalisation      */
  OLC_STAGE_BACKTRANSFORM = 9, /* mixed precision: reflector back-transform and X = U^-1 Z */
  OLC_STAGE_SPLIT = 10,        /* mixed precision: FP64-accurate split products */
  OLC_NUM_STAGES = 11
} olc_stage_t;
int olc_profile_enable(olc_context_t* ctx, int on);
int olc_profile_reset(olc_context_t* ctx);
int olc_profile_read(olc_context_t* ctx, int stage, int64_t* launches, double* ms);
/* Algorithmic work of a stage since the last reset: tensor-core flops issued
 * (the split and FP32-accurate products count every BF16 multiply-add) and
 * the streamed bytes of the HBM-bound kernels (tridiagonalisation: the
 * trailing triangle read once per step, and the lower triangles the
 * between-panel updates read and write). */
int olc_profile_read_work(olc_context_t* ctx, int stage, double* flops, double* bytes);
/* Kernels of this library launched so far in the process (all contexts). */
int64_t olc_launch_count(void);

/* Allocation-free variant of the generalised eigen-solve, for callers that
 * may not allocate device memory once their SCF loop runs: a host program
 * that reserves all device memory for its own pool at start-up, or a
 * framework that owns the device allocator and does not let libraries call
 * cudaMalloc/cudaFree.  This entry point has no counterpart in the reference.
 *
 * Same result as olc_solve_zhegv for n <= 64 (the batched in-shared-memory
 * solver), but needs no context and allocates nothing: every pointer is
 * DEVICE memory supplied by the caller -- packed_h / packed_s [2, n(n+1)/2, nk],
 * eigenvalues [num_states, nk], vectors [n, num_states, nk] (may be NULL),
 * info [nk] (LAPACK-style codes, written by the kernel).  The unpacked
 * working copies live in one 16 MiB device array that every GPU loading the
 * library holds until exit, so nk * n * n must not exceed 524288; larger
 * requests are rejected with OLC_ERR_ARG and a message.
 *
 * The first call on a device looks up that array's device address (with
 * the device current); make that first call before any stream capture.
 * The address is kept per device ordinal for the life of the process: it
 * is not valid after cudaDeviceReset, nor under a second, non-primary
 * context on the same device.
 * Work is queued on `stream` (NULL = legacy stream) and not synchronised.
 * Calls share the array and every call overwrites all of the part it uses,
 * so nothing is carried over between calls, but calls that overlap on the
 * GPU (different streams, or concurrent host threads) race on it. */
int olc_solve_zhegv_noalloc(int n, int nk, const double* packed_h, const double* packed_s,
                            int num_states, double* eigenvalues, double* vectors,
                            int32_t* info, void* stream);

/* Layout-identical raw writers of the reference's HDF5 datasets (no libhdf5
 * is linked).  Every dataset becomes <root>/<group>/<name>.bin with its
 * elements in the dataset's Fortran order as little-endian binary64, and
 * <root>/manifest.json lists path, dims (Fortran order) and type.
 *
 * olc_write_setup_integrals replaces the integral writes of setup-temp.hdf5
 * (hdf5SetupIntg.F90:86-222; integrals.F90:2693, 2826-2840): for every k,
 * /atomIntgGroup/atomOverlap/%07d, atomKEOverlap/%07d, atomNucOverlap/%07d,
 * atomMVOverlap/%07d (rel = 1) and atomPotOverlap/%07d/%07d (k, term), each
 * (2, vale_dim(vale_dim+1)/2)
 * upper-packed orthogonalised values.  Needs olc_scf_prepare(...,
 * OLC_FORM_STORED).
 *
 * olc_write_eigen replaces the eigen writes of main-temp.hdf5
 * (secularEqn.F90:232-270, hdf5MainEval.f90:60-81, hdf5MainEvec.F90:81-119):
 * /eigenValues/%07d%07d (k, spin) of (num_states) and, when vectors != NULL,
 * /eigenVectors/real%07d%07d and imag%07d%07d of (vale_dim, num_states).
 * eigenvalues[num_states, nk] and vectors[vale_dim, num_states, nk] complex
 * are HOST arrays, as olc_scf_iteration returns them. */
int olc_write_setup_integrals(olc_context_t* ctx, const char* root);
int olc_write_eigen(const char* root, int num_kpoints, int spin, int num_states, int vale_dim,
                    const double* eigenvalues, const double* vectors);

/* makeValenceRho for one SCF iteration (src/olcao/valeCharge.F90:34-420;
 * matrixElementMult, src/olcao/matrixSubs.F90:10-53): the valence density
 *   rho_s(k) = sum_n f(n,k,s) x_n x_n^H
 * over the states with sum_s |f(n,k,s)| >= 1e-8 (smallThresh), for spin = 2
 * turned into (up + down, up - down), and its element-wise traces with the
 * prepared operators, summed over k:
 *   traces[3 + rel + pot_dim, spin] = chargeDensityTrace, nucPotTrace,
 *   kineticEnergyTrace, massVelocityTrace (rel = 1 only), potRho(1..pot_dim)
 *   of each spin column (column 1 total, column 2 difference when spin = 2).
 * occupation[num_states, nk, spin] (structuredElectronPopulation: occupation
 * times k-point weight) and eigenvalues[num_states, nk, spin] are HOST
 * arrays; vectors[vale_dim, num_states, nk, spin] complex128 is DEVICE memory
 * (olc_scf_iteration's vectors, one block per spin channel).
 * electron_energy[spin] (HOST, may be NULL; needs eigenvalues) receives
 * sum f * lambda per channel (electronEnergy).  rho_packed (DEVICE, may be
 * NULL) receives packedValeValeRho of every k: [2, packed_len, nk, spin].
 * Needs olc_scf_prepare; with OLC_FORM_FUSED the operators are recomputed
 * one at a time (an integral pass each), with OLC_FORM_STORED the resident
 * ones are read. */
int olc_make_valence_rho(olc_context_t* ctx, int num_states, int spin,
                         const double* occupation, const double* eigenvalues,
                         const double* vectors, double* traces,
                         double* electron_energy, double* rho_packed);

/* populateStates (src/olcao/populate.F90:132-578): occupations of the
 * eigenstates, host arrays only (no context).  eigenvalues[num_states, nk,
 * spin] (Hartree), kpoint_weights[nk] (kPointWeight; each state holds
 * weight / spin electrons).  The states are sorted as the reference sorts
 * them (its merge, ties included), filled up to num_electrons, and the
 * charge of the highest occupied level is spread over the states within
 * 1e-8 Ha of it; with thermal_sigma != 0 (Hartree) the Fermi energy is then
 * found by the reference's bisection with the smeared step function cut at
 * +-max_thermal_range, starting fermi_search_limit (Hartree) outside the
 * highest occupied and the next state.  Writes occupation[num_states, nk,
 * spin] (structuredElectronPopulation, the input of olc_make_valence_rho)
 * and, if not NULL, the highest occupied (Fermi) energy.  XANES core holes
 * are not handled.  OLC_ERR_ARG when the states cannot hold num_electrons. */
int olc_populate_states(int num_states, int num_kpoints, int spin, const double* eigenvalues,
                        const double* kpoint_weights, double num_electrons, double thermal_sigma,
                        double fermi_search_limit, double max_thermal_range,
                        double* occupation, double* occupied_energy);

/* Primitive-level entry (testing and integration checks): one call of the
 * generated primitives (gaussIntegrals.f90) for a batch of inputs on the
 * device.  kind: 1 overlap2CIntg, 2 kinetic2CIntg, 3 nuclear3CIntg,
 * 4 electron3CIntg, 5 massvel2CIntg, 6 / 7 / 8 the x / y / z component of
 * momentum2CIntg (gaussIntegrals.f90:23041-39068, <a| d/dr |b>).
 * in[n*12] = (a1,a2,a3,Ax,Ay,Az,Bx,By,Bz,Cx,Cy,Cz),
 * lmalpha[n*2]; out[n*256] = sh(16,16) column-major (host arrays). */
int olc_primitive_batch(int kind, int n, const double* in,
                        const int32_t* lmalpha, double* out);

#ifdef __cplusplus
}
#endif

#endif /* OLCAO_GPU_H */
