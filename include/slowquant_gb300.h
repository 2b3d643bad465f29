/*
 * slowquant_gb300.h -- C ABI of the GB300 integral / Fock-build library.
 *
 * Every pointer inside the structs and every array argument is DEVICE memory
 * owned by the caller, unless the comment says "host".  Every entry point is
 * asynchronous on the given CUDA stream (a cudaStream_t passed as void*; NULL
 * is the legacy default stream) and returns an int status:
 *   SQ_OK (0) success, or one of the SQ_ERR_* codes below;
 * sq_last_error() returns a human-readable message for the calling thread's
 * last failure.  No entry point allocates device memory except where stated.
 *
 * The Python package (slowquant_gb300) binds these through ctypes and keeps
 * the reference's entry points (SlowQuant, _Integral, run_hartree_fock, DIIS)
 * on top of them.  Paths in the comments are relative to the SlowQuant
 * project.
 */
#ifndef SLOWQUANT_GB300_H
#define SLOWQUANT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SQ_OK 0
#define SQ_ERR_ARG 1          /* null pointer, bad size or inconsistent description */
#define SQ_ERR_UNSUPPORTED 2  /* angular momentum beyond the compiled kernels */
#define SQ_ERR_CUDA 3         /* CUDA launch or runtime error */
#define SQ_ERR_NONFINITE 4    /* NaN or Inf found in an output */

#define SQ_MAX_L 3            /* highest shell angular momentum (f) of the ERI / J-K kernels */
#define SQ_MAX_QCLASS 55      /* quartet classes for l <= SQ_MAX_L: 10 pair classes -> 55;
                                 classes 0-20 hold s, p, d shells only */
#define SQ_MAX_L_GRAD 3       /* highest shell angular momentum of the gradient kernels (f) */

/* Boys-function grid, T_k = k / SQ_BOYS_STEP_INV, k < SQ_BOYS_NGRID.
 * FP64 table (SQ_BOYS_TAB64_SIZE doubles):
 *   [0, NGRID*NCOL): F_m(T_k) at [k*NCOL + m], m < NCOL-1; column NCOL-1 = exp(-T_k);
 *   [SQ_BOYS_TAY64_OFF, ...): Taylor coefficients F_{m+j}(T_k)/j! at
 *     [(m*NGRID + k)*8 + j], j < 7, m < 15; block m = 15 holds exp(-T_k)/j!.
 *   [SQ_BOYS_HI64_OFF, ...): high-order grid for the classes with f shells,
 *     F_m(T_k) at [k*HI_NCOL + m], m < HI_NCOL-1, k < SQ_BOYS_HI_NGRID; column
 *     HI_NCOL-1 = exp(-T_k).  Same step; tabulated to SQ_BOYS_HI_TMAX.
 * FP32 table (SQ_BOYS_TAB32_SIZE floats): the same F grid, then
 *   [SQ_BOYS_TAY32_OFF + (m*NGRID + k)*4 + j], j < 4, and the fifth
 *   coefficient (j = 4) at [SQ_BOYS_TAY32_5_OFF + m*NGRID + k], then the
 *   double-float Taylor rows of the df64 kernels: 12 floats per (m, k) at
 *   [SQ_BOYS_DF_OFF + (m*NGRID + k)*12]: coefficients 0-3 as (hi, lo) pairs,
 *   4-6 as floats, one pad. */
#define SQ_BOYS_NGRID 580
#define SQ_BOYS_STEP_INV 16
#define SQ_BOYS_NCOL 16
#define SQ_BOYS_TMAX 36.0
#define SQ_BOYS_TAY64_OFF (SQ_BOYS_NGRID * SQ_BOYS_NCOL)
#define SQ_BOYS_HI_NGRID 968
#define SQ_BOYS_HI_NCOL 24
#define SQ_BOYS_HI_TMAX 60.0
#define SQ_BOYS_HI64_OFF (SQ_BOYS_TAY64_OFF + 16 * SQ_BOYS_NGRID * 8)
#define SQ_BOYS_TAB64_SIZE (SQ_BOYS_HI64_OFF + SQ_BOYS_HI_NGRID * SQ_BOYS_HI_NCOL)
#define SQ_BOYS_TAY32_OFF (SQ_BOYS_NGRID * SQ_BOYS_NCOL)
#define SQ_BOYS_TAY32_5_OFF (SQ_BOYS_TAY32_OFF + 16 * SQ_BOYS_NGRID * 4)
#define SQ_BOYS_DF_OFF (SQ_BOYS_TAY32_5_OFF + 16 * SQ_BOYS_NGRID)
#define SQ_BOYS_TAB32_SIZE (SQ_BOYS_DF_OFF + 16 * SQ_BOYS_NGRID * 12)

/* Precision of one ERI / J-K launch. */
#define SQ_FP64 0             /* all arithmetic in FP64 */
#define SQ_FP32 1             /* FP32 integral arithmetic, Boys downward recursion in FP64 */
#define SQ_FP32_BOYS32 2      /* FP32 integral arithmetic and FP32 Boys function */
#define SQ_FP64_PRIM 3        /* FP64 with primitive-level precision (sq_jk_prim only): primitive
                                 quartets with q_ij q_kl below a bound run as in SQ_FP32 */
#define SQ_DF64 4             /* double-float arithmetic on the FP32 pipe (sq_jk_df only), with the
                                 same primitive-level split as SQ_FP64_PRIM */

/* Contracted Cartesian Gaussian shells of one molecule (device arrays).
 * Replaces the per-shell Python objects of slowquant/molecule/moleculeclass.py:269-301. */
typedef struct sq_basis {
    int nshell;
    int nbf;
    int natom;
    int nprim_total;
    const double *center;      /* [nshell][3], bohr */
    const int *l;              /* [nshell] angular momentum */
    const int *nprim;          /* [nshell] */
    const int *prim_off;       /* [nshell] first primitive of the shell */
    const int *bf_off;         /* [nshell] first basis function of the shell */
    const double *exps;        /* [nprim_total] Gaussian exponents */
    const double *coefs;       /* [nprim_total] contraction coefficient x the component-independent
                                  part of the normalisation; the per-component factor
                                  1/sqrt((2x-1)!!(2y-1)!!(2z-1)!!) is applied by the kernels */
    const double *atom_xyz;    /* [natom][3], bohr */
    const double *atom_charge; /* [natom] */
    const int *shell_atom;     /* [nshell] atom that carries each shell (used by the gradient kernels) */
    /* Batches of independent molecules (all NULL / 0 for one molecule): the
     * n x n matrices (D, J, K, S, T, V) of molecule i are packed blocks;
     * element (mu, nu) of the molecule that owns shells s, t lives at
     * mat_base[s] + (bf_off[s] + a) * mat_ld[s] + bf_off[t] + b, with bf_off
     * molecule-local; mat_total is the packed length.  The one-electron kernel
     * sums the nuclear attraction over atoms atom_begin[s] <= A < atom_end[s]. */
    const long long *mat_base; /* [nshell] */
    const int *mat_ld;         /* [nshell] */
    long long mat_total;
    const int *atom_begin;     /* [nshell] */
    const int *atom_end;       /* [nshell] */
} sq_basis;

/* Shell pairs and their primitive-pair (Hermite) data.  The caller fills the
 * index arrays and allocates the data arrays; sq_pair_prep writes them. */
typedef struct sq_pairs {
    int npair;
    int nprimpair;
    const int *shells;         /* [npair][2] shells (a, b) with l[a] >= l[b] */
    const int *pp_off;         /* [npair+1] primitive-pair offsets */
    const long long *herm_off; /* [npair] offset of the pair's first Hermite E value */
    double *prim;              /* [nprimpair][8]: p, Px, Py, Pz, U, 0, 0, 0 (U = c_a c_b exp(-mu AB^2) / p) */
    double *herm;              /* Hermite-expanded E^{ab}_{tuv}, x per-component normalisation */
    float *prim32;             /* optional FP32 copy of prim (NULL: not written) */
    float *herm32;             /* optional FP32 copy of herm */
    const double *pq;          /* optional [nprimpair] Schwarz factor sqrt((ij|ij)) of every primitive
                                  pair (NULL: unknown); sq_slots_fill copies it into prim32v */
} sq_pairs;

/* Slot layout of the pair data for the J/K kernels.  Pairs are renumbered in
 * group order (a group = same pair class and primitive counts, sorted by
 * descending Schwarz factor); slot s holds pair pair[s].  Primitive-pair data
 * are stored field-major with the slots of one group fastest, so threads that
 * work on consecutive slots of a group load consecutive addresses:
 *   field f of primitive pair k of slot s: prim[f * npp_total + pbase[s] + k * pstride[s]]
 *   Hermite value e of primitive pair k:   herm[hbase[s] + (k * E + e) * pstride[s]]
 * (E = values per primitive pair of the slot's class, f < 5: p, Px, Py, Pz, U).
 * The caller fills the index arrays and allocates the data arrays;
 * sq_slots_fill copies them from sq_pairs. */
typedef struct sq_slots {
    int nslot;
    long long npp_total;
    long long nherm_total;
    const int *pair;           /* [nslot] */
    const int *npp;            /* [nslot] primitive pairs of the slot */
    const int *pbase;          /* [nslot] */
    const int *pstride;        /* [nslot] */
    const long long *hbase;    /* [nslot] */
    double *prim;              /* [5][npp_total] */
    double *herm;              /* [nherm_total] */
    float *prim32;             /* optional FP32 copies (NULL: not written) */
    float *herm32;
    /* optional primitive-pair selection (NULL: the first npp[s] primitive pairs
     * of the pair): primitive k of slot s is primitive pair
     * prim_src[prim_src_off[s] + k] of the pair's table (i * nprim_b + j). */
    const int *prim_src;
    const long long *prim_src_off; /* [nslot] */
    /* optional sub-slots (NULL: every slot is whole).  sub[s] = 0 for a whole
     * slot; (k << 16) | S for chunk k of S of a slot's primitive pairs (its
     * npp/pbase/hbase then describe that chunk; pair[s] is the parent's pair).
     * Only J/K quartet lists may name sub-slots (bra or ket entries): J and K
     * are linear in the integrals, so the partial quartets add up to the whole.
     * Dense-tensor, Schwarz and gradient lists must name whole slots. */
    const int *sub;
    /* Per-slot descriptor read by the per-thread J/K kernels (required by
     * sq_jk / sq_jk_multi / sq_jk_prim / sq_jk_noalloc; written by
     * sq_slots_describe for all nslot slots): desc[8 s + 0..7] = npp, pbase,
     * pstride, hbase (below 2^31), first basis function of the pair's shell a
     * and of shell b (local to the slot's molecule), pair index with bit 30
     * set when a == b, and the leading dimension of the molecule's n x n
     * matrices.  Two 16-byte loads per slot replace the chain
     * slot -> pair -> shells -> offsets. */
    int *desc;
    /* [nslot] offset of the slot molecule's matrix block in a packed batch,
     * written by sq_slots_describe from basis->mat_base (NULL for one
     * molecule: offset 0). */
    long long *mbase;
    /* Packed FP32 primitive data of the per-thread FP32 J/K kernels (required
     * for FP32 launches; written by sq_slots_fill): 8 floats per primitive
     * pair at prim32v[8 (pbase + k pstride) + f], f = p, Px, Py, Pz, U, the
     * primitive Schwarz factor (0 when pairs->pq is NULL), 0, 0. */
    float *prim32v;
    /* Double-float copies for SQ_DF64 launches (sq_jk_df; written by
     * sq_slots_fill when non-NULL): every value v as the float pair (hi, lo),
     * hi = (float)v, lo = (float)(v - hi); primdf holds 2 * 5 * npp_total floats
     * laid out like prim (pair index f * npp_total + i), hermdf 2 * nherm_total
     * floats laid out like herm. */
    float *primdf;
    float *hermdf;
} sq_slots;

/* Shell-quartet work list: device array of (bra pair, ket pair) index pairs,
 * grouped by quartet class; class_off (host) delimits each class segment.
 * Quartet class of pair classes cb >= ck is cb*(cb+1)/2 + ck. */
typedef struct sq_quartets {
    long long nquartet;
    const int *pairs;                        /* [nquartet][2] */
    long long class_off[SQ_MAX_QCLASS + 1];  /* host */
} sq_quartets;

/* Library version and last error. */
int sq_version(void);
const char *sq_last_error(void);

/* Process-wide tuning options (no reference counterpart).
 * SQ_OPT_GENERIC_MIN_L: quartet classes with la+lb+lc+ld >= value run on the
 * generic warp-cooperative kernel, the others on the per-class unrolled
 * kernels (default 5; SQ_FP32 launches of the classes up to (dd|ds) stay
 * unrolled unless the value is 0, which sends every class to the generic
 * kernel). */
#define SQ_OPT_GENERIC_MIN_L 1
/* SQ_OPT_JK_STREAMS: the J/K class launches of one call are spread over this
 * many library-owned streams (1..16, default 8), forked from and joined back
 * into the caller's stream with events, so that one class's tail overlaps the
 * next class; 1 launches everything on the caller's stream.  Successive calls
 * take the next streams of a pool of 16, so calls issued concurrently from
 * different caller streams run side by side.  The pool (streams and events,
 * kept until the process exits) is created by the first multi-stream J/K call
 * on each device: make that call outside any stream capture. */
#define SQ_OPT_JK_STREAMS 2
/* SQ_OPT_FP64_UNROLLED_HIGH: bit mask over quartet classes; a set bit runs
 * that class's FP64 J/K launches on its per-thread kernel where one exists
 * (classes 12-18, (dp|pp) to (dd|ds)), a clear bit on the generic warp
 * kernel.  Default: classes 12-18. */
#define SQ_OPT_FP64_UNROLLED_HIGH 3
/* SQ_OPT_GRAD_THREAD: 1 (default) runs the gradient of the light classes
 * ((ss|ss), (ps|ss), (ps|ps), (pp|ss), (pp|ps), (ds|ss), (ds|ps), (dp|ss))
 * one quartet per thread, 0 one quartet per warp like the other classes. */
#define SQ_OPT_GRAD_THREAD 4
/* SQ_OPT_DF_CLASSES: which classes of an SQ_DF64 launch (sq_jk_df) run on
 * their double-float kernel; the others run as in sq_jk_prim (FP64, with the
 * primitive split where the class has it).  -1 (default): the measured
 * policy -- always for (ss|ss), (ps|ss), (ps|ps), (pp|ss), (ds|ss), (ds|ps),
 * (dp|ss), (dd|ss), (dd|ps); for (pp|ps), (pp|pp), (ds|pp), (ds|ds), (dp|ps)
 * when the launch holds at least 512 quartets per SM; never for (dp|pp),
 * (dp|ds), (dp|dp), (dd|pp), (dd|ds), whose double-float kernels spill more
 * than their FP64 ones.  A mask >= 0 over classes 0-18 selects exactly the
 * set bits, whatever the launch length. */
#define SQ_OPT_DF_CLASSES 5
int sq_set_option(int key, long long value);
long long sq_get_option(int key);

/* Launch shape ("tile") of the J/K kernels of one quartet class and precision
 * (no reference counterpart), set by the autotuner (slowquant_gb300.autotune):
 * threads per block (32..128 for the per-quartet kernels; the generic warp
 * kernel always runs 4 warps) and the grid cap in blocks (quartets beyond
 * blocks x threads are taken by a grid-stride loop).  threads = 0 restores
 * the built-in default. */
int sq_set_launch_config(int qclass, int precision, int threads, long long max_blocks);

/* Fill the FP64 Boys table (SQ_BOYS_TAB64_SIZE doubles) and, if
 * table32 != NULL, the FP32 table (SQ_BOYS_TAB32_SIZE floats).  Replaces nothing: the reference
 * evaluates boys_function by series on every call
 * (slowquant/molecularintegrals/integralfunctions.py:74-97). */
int sq_boys_table(double *table64, float *table32, void *stream);

/* F_0..F_{n_max}(z[i]) for nz arguments -> out[nz][n_max+1].
 * mode 0: the tabulated function the J/K kernels of classes 0-20 use (n_max <= 8);
 * mode 1: the reference's piecewise formula that the dense-tensor and Schwarz
 * kernels use (n_max <= 22); mode 2: the high-order table of the J/K kernels of
 * the classes with f shells (n_max <= 16).  Test hook for boys_function
 * (integralfunctions.py:74-97). */
int sq_boys(int n_max, const double *z, long long nz, const double *table64, int mode, double *out, void *stream);

/* F_0..F_{n_max}(z[i]) (n_max <= 8) as the double-float J/K kernels evaluate
 * them (Taylor rows at SQ_BOYS_DF_OFF of table32, downward recursion, all in
 * float pairs), returned as hi + lo in FP64 -> out[nz][n_max+1].  Test hook. */
int sq_boys_df(int n_max, const double *z, long long nz, const float *table32, double *out, void *stream);

/* Primitive-pair data for every pair in `pairs`: P, p, U and the Hermite
 * expansion coefficients of expansion_coefficients
 * (integralfunctions.py:9-71), times the per-component normalisation of
 * Shell.normalization (moleculeclass.py:292-299). */
int sq_pair_prep(const sq_basis *basis, sq_pairs *pairs, void *stream);

/* q[P] = sqrt(max over the (ab|ab) block) for every diagonal quartet (P, P)
 * listed in `diagonal`: the shell-pair Cauchy-Schwarz matrix of
 * get_cauchy_schwarz_matrix (slowquant/molecularintegrals/electronrepulsion.py:
 * 300-339). */
int sq_schwarz(const sq_basis *basis, const sq_pairs *pairs, const sq_quartets *diagonal, const double *table64,
               double *q, void *stream);

/* Copy the primitive-pair data of `pairs` into the slot layout.  Replaces
 * nothing in the reference (it recomputes pair data per quartet,
 * electronrepulsion.py:206-237). */
int sq_slots_fill(const sq_basis *basis, const sq_pairs *pairs, sq_slots *slots, void *stream);

/* Fill slots->desc (and slots->mbase for a packed batch basis) for all
 * nslot slots, sub-slots included.  No counterpart in the reference. */
int sq_slots_describe(const sq_basis *basis, const sq_pairs *pairs, sq_slots *slots, void *stream);

/* Dense ERI tensor V[nbf^4] (C order) from the quartets of `quartets` (slot
 * ids when slots != NULL, else pair ids), each block scattered to its eight
 * index permutations: the output of electron_repulsion_integral_driver
 * (electronrepulsion.py:11-104).  V must be zeroed by the caller. */
int sq_eri_dense(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
                 const double *table64, double *V, void *stream);

/* Integral-direct Coulomb / exchange build: for the unique quartets of
 * `quartets` (slot ids of `slots`), accumulate into Jacc/Kacc ([nbf][nbf], FP64, caller zeroes)
 * so that sym(Jacc) = J = einsum("pqrs,sr->pq", ERI, D) and
 * sym(Kacc) = K = einsum("psqr,sr->pq", ERI, D), the two einsums of
 * run_hartree_fock (slowquant/hartreefock/hartreefock_in_memory.py:55-56).
 * precision is SQ_FP64, SQ_FP32 or SQ_FP32_BOYS32; FP32 launches accumulate
 * each quartet's FP32 contributions into the FP64 Jacc/Kacc.  D32 is caller
 * scratch of nbf*nbf floats that FP32 launches fill with (float)D (unused,
 * may be NULL, for SQ_FP64); FP32 launches need pairs->prim32/herm32 and
 * table32. */
int sq_jk(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
          const double *table64, const float *table32, const double *D, float *D32, double *Jacc, double *Kacc,
          int precision, void *stream);

/* J and K from a stored ERI tensor V[nbf^4] (C order): J[p][q] =
 * sum_rs V[p][q][r][s] D[s][r] and K[p][q] = sum_rs V[p][s][q][r] D[s][r], the
 * two einsums of run_hartree_fock when it is given the tensor
 * (hartreefock_in_memory.py:55-56), in one pass over V.  J and K ([nbf][nbf])
 * are overwritten. */
int sq_jk_dense(int nbf, const double *V, const double *D, double *J, double *K, void *stream);

/* Several densities per integral evaluation (the two spin densities of
 * unrestricted HF, slowquant/hartreefock/unrestricted_hartreefock_in_memory.py:69-74,
 * which the reference contracts four times with the stored tensor): like
 * sq_jk, but D, D32, Jacc and Kacc each hold nd consecutive matrices of
 * mat_total elements (nbf*nbf without packing), and every quartet's
 * integrals are computed once and digested into J_i, K_i for every D_i. */
int sq_jk_multi(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
                const double *table64, const float *table32, int nd, const double *D, float *D32, double *Jacc,
                double *Kacc, int precision, void *stream);

/* Primitive-level precision for the large-bound quartets of a mixed build
 * (no counterpart in the reference).  Like sq_jk with SQ_FP64, except that in
 * the classes with per-thread kernels (la+lb+lc+ld <= 4 except (dd|ss), and
 * (fs|ss), (fs|ps), (fp|ss)) every primitive quartet whose primitive Schwarz
 * bound q_ij q_kl is below prim_tau is evaluated in FP32 with the FP64 Boys
 * recursion, summed in FP32 per bra primitive pair and added into the FP64
 * block before the FP64 digestion.  q comes from slots->prim32v (written by
 * sq_slots_fill from pairs->pq, which must be set); FP32 slot data, herm32
 * and table32 are required.  The other classes run plain FP64. */
int sq_jk_prim(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
               const double *table64, const float *table32, const double *D, double *Jacc, double *Kacc,
               double prim_tau, void *stream);

/* Double-float J/K build (no counterpart in the reference).  Like sq_jk_prim,
 * except that the classes (ss|ss) to (dd|ds) carry every FP64 quantity as a
 * pair of floats (hi + lo, about 46 significant bits) and do all their
 * arithmetic on the FP32 pipe, which GB300 runs at about 60 times its FP64
 * rate; Boys values come from the double-float rows of table32
 * (SQ_BOYS_DF_OFF).  prim_tau splits as in sq_jk_prim (0: every primitive
 * quartet in double-float; pairs->pq is then not needed).  Ddf is caller scratch of 2 * nbf * nbf floats
 * (mat_total pairs for a packed basis) that the call fills with D as
 * double-float pairs; slots->primdf and slots->hermdf must be written (by
 * sq_slots_fill).  The classes without a double-float kernel run as in
 * sq_jk_prim.  J/K accumulate in FP64. */
int sq_jk_df(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
             const double *table64, const float *table32, const double *D, float *Ddf, double *Jacc, double *Kacc,
             double prim_tau, void *stream);

/* 1 when an SQ_DF64 launch of quartet class qclass holding nquartets list
 * entries runs on the class's double-float kernel (option SQ_OPT_DF_CLASSES),
 * else 0.  Host-only query. */
int sq_df_class(int qclass, long long nquartets);

/* J/K build for callers that cannot allocate device memory.  No counterpart
 * in the reference (it has no device code).  Same arguments and results as
 * sq_jk, minus D32: the FP32 density scratch that FP32 launches need lives in
 * a fixed array inside this library (SQ_NOALLOC_MAX_ELEMS floats, 4 MiB, held
 * on every GPU that loads the library until the process exits).  It serves
 * hosts that own all device memory, streams whose capture mode forbids
 * allocation, and loops that cannot afford cudaMalloc's synchronisation.
 * The limit is in matrix elements: nbf > SQ_NOALLOC_MAX_NBF, or a density of
 * more than SQ_NOALLOC_MAX_ELEMS elements (mat_total of a packed batch basis,
 * sum_i n_i^2, whatever its nbf), is rejected with SQ_ERR_ARG before any
 * device work.  Every call looks up (first call on a device) or reuses the
 * array's device address; make the first call on each device before any
 * stream capture.  Calls share the array, so calls that overlap on the GPU
 * race and must be serialised by the caller; each FP32 call overwrites the
 * elements it reads before reading them.  Allocates nothing. */
#define SQ_NOALLOC_MAX_NBF 1024
#define SQ_NOALLOC_MAX_ELEMS (SQ_NOALLOC_MAX_NBF * SQ_NOALLOC_MAX_NBF)
int sq_jk_noalloc(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
                  const double *table64, const float *table32, const double *D, double *Jacc, double *Kacc,
                  int precision, void *stream);

/* F = H + J - K/2 with J = (Jacc + Jacc^T)/2, K = (Kacc + Kacc^T)/2
 * (hartreefock_in_memory.py:57); J and K may be NULL. */
int sq_fock_build(int nbf, const double *H, const double *Jacc, const double *Kacc, double *F, double *J,
                  double *K, void *stream);

/* One-electron matrices S, T, V ([nbf][nbf]; any may be NULL): overlap
 * (multipole.py:48-135 with moment 0), kinetic energy (kineticenergy.py:42-133)
 * and nuclear attraction (nuclearattraction.py:47-135). */
int sq_one_electron(const sq_basis *basis, const double *table64, double *S, double *T, double *V,
                    void *stream);

/* Multipole integral matrix M[nbf][nbf] = <a| (x-Cx)^ex (y-Cy)^ey (z-Cz)^ez |b>
 * (multipole_integral_driver, slowquant/molecularintegrals/multipole.py:10-135,
 * with the Hermite multipole recursion of integralfunctions.py:151-183).
 * order (host, [3]) = (ex, ey, ez), each 0..16; origin (host, [3]) = C in the
 * coordinates of basis->center.  order (0,0,0) is the overlap. */
int sq_multipole(const sq_basis *basis, const int *order, const double *origin, double *M, void *stream);

/* Expand per-bra tasks into the flat quartet list: task i writes
 * (bra[i], ket_list[ket_start[i] + k]) for k < count[i] at out[offset[i] + k],
 * or (bra[i], ket_start[i] + k) when ket_list is NULL (slot ids).  offset is
 * the exclusive prefix sum of count.  Replaces the shell-quartet loops and the
 * Schwarz skip of electronrepulsion.py:32-49. */
int sq_quartets_expand(long long ntask, const int *bra, const int *ket_start, const int *count,
                       const long long *offset, const int *ket_list, int *out_pairs, long long nquartet,
                       void *stream);

/* RHF nuclear gradient, two-electron part (no reference counterpart: the
 * reference has no gradients).  For every unique quartet of `quartets` (slot
 * ids) the derivative integrals are formed on the fly and contracted with the
 * two-particle density of D, never stored:
 *   grad[atom][xyz] += (m/2) sum_abcd Gamma'_abcd d(ab|cd)/dR,
 *   Gamma'_abcd = D_ab D_cd - (D_ac D_bd + D_ad D_bc)/4,  m = permutational weight.
 * grad is [natom][3] FP64, accumulated (caller zeroes).  FP64 arithmetic. */
int sq_grad_2e(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots, const sq_quartets *quartets,
               const double *table64, const double *D, double *grad, void *stream);

/* RHF nuclear gradient, one-electron part: grad += sum_ab D_ab dH_ab/dR -
 * sum_ab W_ab dS_ab/dR (kinetic energy, nuclear attraction including the
 * derivative with respect to each nucleus, overlap), for D, W [nbf][nbf]. */
int sq_grad_1e(const sq_basis *basis, const double *table64, const double *D, const double *W, double *grad,
               void *stream);

/* One pass of the AO -> MO transformation (slowquant/molecularintegrals/
 * integralfunctions.py:186-211, which contracts with numpy einsum):
 *   out[l][r] = sum_{d < n} G[r][d] C[d][l],   r < rows, l < m,
 * G rows x n and C n x m row-major, out m x rows.  Transforming the last index
 * and moving it to the front, four passes turn g[a][b][c][d] into
 * g[i][j][k][l] (rows = n^3, m n^2, m^2 n, m^3) and two turn h into C^T h C.
 * out must not alias G.  FP64 arithmetic. */
int sq_ao2mo_rotate(long long rows, int n, int m, const double *G, const double *C, double *out, void *stream);

/* Batched symmetric eigensolver (replaces the per-molecule numpy eigh of the
 * SCF step, slowquant/hartreefock/hartreefock_in_memory.py:63-66, when many
 * molecules run at once).  Matrix i is dims[i] x dims[i] (1..128), row-major
 * at A + offsets[i]; its eigenvalues go to W + w_offsets[i] in ascending order
 * and the eigenvectors, as columns, to V + offsets[i].  Cyclic Jacobi, one
 * CTA per matrix; stops when ||offdiag||_F <= tol ||A||_F or after max_sweeps
 * sweeps.  sweeps (nullable, [nmat]) receives the sweeps used (-1: dims[i]
 * outside 1..max_dim, matrix skipped).  max_dim = max(dims) (<= 128). */
int sq_batched_eigh(int nmat, const long long *offsets, const int *dims, int max_dim, const double *A, double *W,
                    double *V, const long long *w_offsets, double tol, int max_sweeps, int *sweeps, void *stream);

/* Arithmetic-pipe probe (no reference counterpart): blocks x 256 threads each
 * run `iters` iterations of 8 independent FMA chains in FP64 (precision
 * SQ_FP64), double-float (SQ_DF64: float pairs, csrc/df64.cuh) or FP32
 * (otherwise), i.e. 16 * iters * 256 * blocks FLOPs; out holds blocks*256
 * elements of that type (8 bytes for SQ_DF64).  Timing it gives the measured
 * FMA peak used as the roofline denominator of the FP64-, double-float- and
 * FP32-bound kernels. */
int sq_fma_probe(int precision, int blocks, int iters, void *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SLOWQUANT_GB300_H */
