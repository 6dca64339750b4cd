/*
 * sbe_gb300.h - C ABI of the GB300 quantum-wire SBE / PSTD library (libsbe_gb300.so).
 *
 * Conventions
 *  - Every entry point returns int: 0 = OK, >0 = error (SBE_ERR_*); the message of
 *    the last error on the calling thread is returned by sbe_last_error().
 *  - All array arguments are DEVICE pointers (cudaMalloc'd or torch CUDA tensors),
 *    contiguous, row-major, at least 16-byte aligned.  Complex numbers are
 *    interleaved (re, im) doubles ("c128").
 *  - A matrix of one wire is Nk x Nk row-major.  The coherence p is stored
 *    [kh][ke] and Heh/Meh are stored [ke][kh], as in the reference.
 *  - Calls are asynchronous on the given stream (a cudaStream_t passed as void*;
 *    NULL = legacy default stream).  Nothing is copied to or from the host.
 *  - No call falls back to the CPU: a missing device or a failed launch is an error.
 *
 * Reference interfaces replaced (rahulranjansah/pulsesuite, src/pulsesuite/PSTD3D):
 *  each declaration cites the function it stands in for.
 */
#ifndef SBE_GB300_H
#define SBE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SBE_OK 0
#define SBE_ERR_ARG 1        /* invalid argument (null pointer, size, flag) */
#define SBE_ERR_UNSUPPORTED 2/* Nk or mode outside what the build supports     */
#define SBE_ERR_OOM 3        /* device allocation failed                        */
#define SBE_ERR_CUDA 4       /* a CUDA runtime/driver call failed               */
#define SBE_ERR_TIMEOUT 5    /* a bounded device-side wait gave up              */

/* Many-body flags (mb.params order, SBEs.py:5004-5022). */
#define SBE_F_OPTICS     (1 << 0)
#define SBE_F_EXCITONS   (1 << 1)
#define SBE_F_EHS        (1 << 2)
#define SBE_F_SCREENED   (1 << 3)
#define SBE_F_PHONON     (1 << 4)
#define SBE_F_DCTRANS    (1 << 5)
#define SBE_F_LF         (1 << 6)
#define SBE_F_FREEPOT    (1 << 7)
#define SBE_F_DIAGDPH    (1 << 8)
#define SBE_F_OFFDIAGDPH (1 << 9)
#define SBE_F_RECOMB     (1 << 10)
#define SBE_F_LORENTZ    (1 << 11)  /* LorentzDelta of mb.params: Lorentzian broadening of the EHs rates */

/* Precision of the RHS contractions. */
#define SBE_PREC_FP64  0  /* plain FP64 SIMT (drop-in path and on-device reference) */
#define SBE_PREC_MIXED 1  /* tcgen05 FP16 hi/lo x3, FP32 accumulate, FP64 state    */

/* One wire: grid and material in SI units (qw.params, SBEs.py:4978-5002). */
typedef struct {
  int nk;            /* k points (even, >= 4)                                  */
  int wire_index;    /* w (1-based) for yw(w) and (-1)^w                       */
  int flags;         /* SBE_F_* bitmask                                        */
  int pad0;
  double L;          /* wire length (m); dkr = pi / L, Nr = 2 Nk + 2           */
  double Delta0;     /* thickness (m)                                          */
  double gap;        /* band gap (J)                                           */
  double me, mh;     /* effective masses (kg)                                  */
  double HO;         /* confinement level spacing (J)                          */
  double gam_e, gam_h, gam_eh;  /* rates (1/s)                                 */
  double epsr;       /* background dielectric constant                         */
  double Oph, Gph;   /* LO phonon frequency and damping (rad/s)                */
  double temp;       /* lattice temperature (K) (phonons.py:22)                */
  double Edc;        /* DC field along the wire (V/m), qw.params (SBEs.py:1317);
                        used by DC transport (SBE_F_DCTRANS)                   */
} SbeWireDesc;

typedef struct SbeCtx SbeCtx;

/* ---- library ------------------------------------------------------------- */
const char* sbe_last_error(void);
int sbe_version(void);
/* Physical constants compiled into the library (CODATA 2022: hbar, e, eps0, me0, kB). */
int sbe_constants(double* out5);

/* ---- context: tables built once on the device in FP64 -------------------- */
/* Replaces SBESolver.__init__ table set-up (SBEs.py:4623-4972): grid, kkp,
 * CoulombModule (coulomb.py:1124-1164), InitializePhonons (phonons.py:55),
 * InitializeDephasing (dephasing.py:472), QWOptics (qwoptics.py:575).        */
int sbe_ctx_create(const SbeWireDesc* wires, int n_wires, void* stream, SbeCtx** out);
int sbe_ctx_destroy(SbeCtx* ctx);
/* The packed buffers group the wires by Nk (ascending; the caller's order within
 * one Nk), so that the wires of one Nk are contiguous (the mixed path's buckets).
 * Per-wire sizes/offsets (elements) of the packed state: out[3*w+0] = Nk,
 * out[3*w+1] = offset of wire w's Nk*Nk block, out[3*w+2] = offset of its Nr block. */
int sbe_ctx_layout(const SbeCtx* ctx, long long* out, long long* total_mat, long long* total_r);
/* Copy one table of wire w into dst (device). which: 0 kr, 1 r, 2 Ee, 3 Eh,
 * 4 V0 (3*Nk: eh, ee, hh by k1-k2 >= 0), 5 Chi1D (2*Nk by |k1-k2|), 6 qe/qh (2*Nk),
 * 7 EP (Nk*Nk), 8 HP (Nk*Nk), 9 window (Nr), 10 dephasing maps (6*Nk*Nk int32),
 * 11 xe/xh (2*Nk), 12 Expikr (c128 Nk*Nr), 13 scalars (16 doubles).          */
int sbe_ctx_table(const SbeCtx* ctx, int w, int which, void* dst, long long nbytes, void* stream);

/* ---- reference pure functions, one wire, FP64 ---------------------------- */
/* SBEs.py:1839 dpdt (p[kh][ke]).                                               */
int sbe_dpdt(int nk, const double* C, const double* D, const double* P, const double* Heh,
             const double* Hee, const double* Hhh, const double* GamE, const double* GamH,
             const double* OffP, double* out, void* stream);
/* SBEs.py:2210 dCdt.                                                           */
int sbe_dCdt(int nk, const double* C, const double* D, const double* P, const double* Heh,
             const double* Hee, const double* Hhh, double* out, void* stream);
/* SBEs.py:2502 dDdt.                                                           */
int sbe_dDdt(int nk, const double* C, const double* D, const double* P, const double* Heh,
             const double* Hee, const double* Hhh, double* out, void* stream);
/* SBEs.py:658 CalcH (VC is Nk*Nk*3 real, [k1][k2][n]; only VC[q][0][n] is read).
 * Having no context, it takes its scratch (3 Nk doubles, 4 Nk complex) from the
 * device's stream-ordered pool (cudaMallocAsync / cudaFreeAsync on stream: no host
 * synchronisation); the batched context path builds H with no allocation.      */
int sbe_calch(int nk, const double* Meh, const double* Wee, const double* Whh, const double* C,
              const double* D, const double* P, const double* VC, const double* Ee,
              const double* Eh, double gap, int excitons, int lf, int freepot, double* Heh,
              double* Hee, double* Hhh, void* stream);

/* ---- per-wire building blocks of one context (FP64) ---------------------- */
/* coulomb.py:1195 CalcScreenedArrays for wire w: VC (Nk*Nk*3) and E1D (Nk*Nk). */
int sbe_screened_arrays(SbeCtx* ctx, int w, const double* ne, const double* nh, double* VC,
                        double* E1D, void* stream);
/* dephasing.py:541/584 CalcGammaE/H from VC (Nk*Nk*3).                        */
int sbe_gamma(SbeCtx* ctx, int w, const double* ne, const double* nh, const double* VC,
              double* GamE, double* GamH, void* stream);
/* dephasing.py:714 OffDiagDephasing2: x (c128 Nk*Nk); De, Dh ((2Nk+1)*Nk), g = [geh, ge, gh]. */
int sbe_offdiag(SbeCtx* ctx, int w, const double* ne, const double* nh, const double* P,
                const double* VC, const double* g3, double* x, double* De, double* Dh,
                void* stream);
/* phonons.py:157/223 MBPE/MBPH: Win/Wout accumulated in place.                 */
int sbe_phonon_rates(SbeCtx* ctx, int w, const double* ne, const double* nh, const double* VC,
                     const double* E1D, double* WinE, double* WoutE, double* WinH,
                     double* WoutH, void* stream);
/* emission.py:94 SpontEmission (Recomb) with the tables of InitializeEmission
 * (emission.py:35, the module's 77 K): Rsp (f64 Nk) at ne, nh (c128 Nk, real parts
 * used) and VC (Nk*Nk*3).  The wire must have SBE_F_RECOMB.                    */
int sbe_spont_emission(SbeCtx* ctx, int w, const double* ne, const double* nh, const double* VC,
                       double* Rsp, void* stream);
/* The per-step statistics of wire w that SBEs.py:5769-5809 appends to
 * dataQW/info.WW.t.dat and dataQW/EP.WW.t.dat, reduced on the device.  C2, D2:
 * the packed middle-level state (ne2 = |C2_kk|, nh2 = |D2_kk|); src: the packed
 * real-space sources (per wire 5 x c128 Nr: Px, Py, Pz, re, rh); Ek: the packed
 * wire-k field (3 x c128 Nr); VC (Nk*Nk*3) or NULL for the last step's screened
 * interaction.  out23 (device): CalcVD e/h (dcfield.py:128), densities 2 sum n / L,
 * TotalEnergy e (with the gap)/h in eV, Temperature e/h (usefulsubs.py:1185-1253),
 * max |FFTG re|, max |FFTG rh| (the reference takes them over its wire-k arrays),
 * GetEDrift (0: SBEs never sets it), momenta 2 hbar sum (ne-nh) k,
 * hbar sum ne k, -hbar sum nh k, CalcI0 (dcfield.py:1110), CalcI0n e and h
 * (:103, real parts; their imaginary parts are 0); then Re iFFTG(Ex, Ey, Ez)[Nr/2]
 * and Re Px, Py, Pz [Nr/2].                                                     */
int sbe_wire_info(SbeCtx* ctx, int w, const double* C2, const double* D2, const double* src,
                  const double* Ek, const double* VC, double* out23, void* stream);
/* SBEs.py:5924-5978 PdotE.w.dat, the wire-grid term of the reference's EPEnergyW:
 * *out (device) = sum_{c = x,y,z} sum_r (Re P_c(r) - P0_c(r)) Re E_c(r) with P_c the
 * packed real-space sources src (5 x c128 Nr per wire), E_c = iFFTG of the packed
 * wire-k field Ek (3 x c128 Nr per wire; usefulsubs.py:2271, the QW2Prop
 * transform of qwoptics.py:775) and P0 (f64 3 x Nr, the caller's history of Re P;
 * NULL: zeros).  The caller applies 0.5 dr area and accumulates.              */
int sbe_wire_pdote(SbeCtx* ctx, int w, const double* Ek, const double* src, const double* P0,
                   double* out, void* stream);
/* dephasing.py:731-740 (MaxOffDiag.e.dat / .h.dat): out4 (device) = max Re De,
 * min Re De, max Re Dh, min Re Dh of wire w's off-diagonal dephasing matrices
 * ([2Nk+1][Nk]) of the last preparation (either path).                        */
int sbe_deph_extrema(SbeCtx* ctx, int w, double* out4, void* stream);
/* coulomb.py:1298/1313 MBCE/MBCH (carrier-carrier scattering, EHs; tables of
 * CalcMBArrays, coulomb.py:367, evaluated on the fly, Lorentzian broadening with
 * SBE_F_LORENTZ in the wire's flags, else Gaussian): Win/Wout accumulated in place.
 * ne, nh c128 Nk (|Re| used); VC (Nk*Nk*3).  precision SBE_PREC_FP64 (the
 * reference's arithmetic) or SBE_PREC_MIXED (FP32, exact integer energy sums).   */
int sbe_carrier_rates(SbeCtx* ctx, int w, const double* ne, const double* nh, const double* VC,
                      double* WinE, double* WoutE, double* WinH, double* WoutH, int precision,
                      void* stream);
/* qwoptics.py:809 QWPolarization3 and 942 QWRho5 (with x 2 e0 ehint/area), real
 * space (before FFTG): Px, Py, Pz, re, rh (c128 Nr).  ne/nh c128 Nk.         */
int sbe_sources(SbeCtx* ctx, int w, const double* P, const double* C, const double* D,
                const double* ne, const double* nh, double* Px, double* Py, double* Pz,
                double* re, double* rh, void* stream);
/* qwoptics.py:667 Prop2QW: spline from the propagation grid RR (n_rr) to the wire
 * grid, window, real part, FFTG.  fields_in: 4 x c128 n_rr (Exx, Eyy, Ezz, Vrr);
 * out: 4 x c128 Nr.  The spline scratch (12 x c128 n_rr) is the context's: the
 * first call and a call with a larger grid than any before allocate it (cudaMalloc;
 * growing it waits for the device), other calls allocate nothing.              */
int sbe_prop2qw(SbeCtx* ctx, int w, const double* RR, int n_rr, const double* fields_in,
                double* out, void* stream);
/* qwoptics.py:717 QW2Prop (real-space sources in): 5 x c128 Nr (Px, Py, Pz, re, rh)
 * -> 5 x c128 n_rr (Pxx, Pyy, Pzz, RhoE, RhoH).  Scratch from the context's arena. */
int sbe_qw2prop(SbeCtx* ctx, int w, const double* RR, int n_rr, const double* src_in,
                double* out, int plasmonics, void* stream);

/* ---- Prop2QW without allocation (no counterpart in the reference) ------------
 * Same arguments and results as sbe_prop2qw, for callers that must not allocate
 * device memory (a host code whose pool owns all device memory, or a loop that
 * must not take the allocator's lock): the scratch is one static device array
 * per CUDA context (each context loads its own copy of the library's module), so
 * nothing is allocated or freed.  Limits: n_rr <= SBE_NOALLOC_MAX_GRID, wire
 * Nr <= SBE_NOALLOC_MAX_NR; larger calls return an error before any launch.
 * Every call looks the array up in the current context (cudaGetSymbolAddress,
 * nothing cached, so a reset or new context is safe); the first call in a
 * context may load the module, so make it before any stream capture.  Calls of
 * one context that overlap in time (other streams or threads) race on the shared
 * scratch; calls on one stream are ordered.                                    */
#define SBE_NOALLOC_MAX_GRID 8192
#define SBE_NOALLOC_MAX_NR 2050
int sbe_prop2qw_noalloc(SbeCtx* ctx, int w, const double* RR, int n_rr,
                        const double* fields_in, double* out, void* stream);

/* ---- the reference time step (leapfrog), all wires of the context -------- */
/* SBEs.py:5612-5820 _sbe_calculator for every wire of ctx.  State: 9 buffers of
 * packed Nk*Nk c128 blocks (YY1..3, CC1..3, DD1..3 in that order in state9[]).
 * Ek: per wire 3 x c128 Nr field in wire k space (FFTG'd Ex, Ey, Ez).
 * src_out: per wire 5 x c128 Nr real-space sources (Px, Py, Pz, re, rh).     */
int sbe_leapfrog_step(SbeCtx* ctx, double* const* state9, const double* Ek, double dt,
                      double* src_out, void* stream);

/* ---- batched RK4 (the GB300 path), all wires ------------------------------- */
/* One RK4 step of dt for every wire: state P, C, D (packed c128), field in wire
 * k space at the step start Ek0 and its change per step dEk (both 3 x c128 Nr per
 * wire; stage fields Ek0 + c dEk).  Relaxation, charge normalisation and the
 * sources of the new state follow (as in the reference step).  precision:
 * SBE_PREC_FP64 or SBE_PREC_MIXED (SBE_ERR_UNSUPPORTED for a context with
 * SBE_F_DCTRANS: the reference's transport leaves C, D non-Hermitian; the mixed
 * path also needs one flag set over the context and every Nk a multiple of 8; the
 * Nk may differ between wires).                                                */
int sbe_rk4_step(SbeCtx* ctx, double* P, double* C, double* D, const double* Ek0,
                 const double* dEk, double dt, int precision, double* src_out, void* stream);
/* A local field uniform along every wire (the local-field drivers of the reference,
 * sbetestprop.py:184-198, whose Prop2QW of a constant field is E FFTG(window),
 * qwoptics.py:667-715): component comp (0 x, 1 y, 2 z) of wire w's Ek0 is e0[w]
 * FFTG(window_w), the others 0; dEk (may be NULL) likewise from de.  e0, de:
 * device arrays of one amplitude (V/m) per wire, in the caller's wire order.     */
int sbe_local_field(SbeCtx* ctx, const double* e0, const double* de, int comp, double* Ek0,
                    double* dEk, void* stream);
/* The coherent RHS of every wire at the given state/field (preparation included),
 * for parity checks.                                                           */
int sbe_rhs(SbeCtx* ctx, const double* P, const double* C, const double* D, const double* Ek,
            int precision, double* dP, double* dC, double* dD, void* stream);

/* ---- CUDA graph of one step (no counterpart in the reference) -------------- */
/* Capture one sbe_rk4_step with the given (fixed) buffers into a CUDA graph on a
 * private stream and instantiate it; *n_kernels receives the number of kernel
 * nodes (the launches of one step).  Call once uncaptured first so that the
 * mixed-precision workspace exists.  Replays read Ek0/dEk and update P, C, D and
 * src_out in place.                                                             */
typedef struct SbeGraph SbeGraph;
int sbe_rk4_graph_create(SbeCtx* ctx, double* P, double* C, double* D, const double* Ek0,
                         const double* dEk, double dt, int precision, double* src_out,
                         SbeGraph** out, long long* n_kernels);
int sbe_graph_launch(SbeGraph* g, void* stream);
int sbe_graph_destroy(SbeGraph* g);

/* ---- tile autotuner of the mixed path (no counterpart in the reference) ------
 * The reference runs its wires one after another (rhoPJ.py:306-343,
 * sbetestprop.py:204-209); here the wires of one Nk form a bucket and each GEMM
 * kind of a stage runs as one persistent launch over all buckets.  sbe_autotune
 * chooses, per bucket, the N tile (256 or 128) of the exchange, commutator and
 * source GEMMs by timing both on the context's workspace, and caches the choice in
 * the JSON file cache_json (NULL: no cache) under a key of the device and the
 * context's (Nk, wires) buckets: a later call with a matching entry loads it and
 * times nothing.  Without a call every GEMM uses the 256 tile.  Synchronises the
 * device; not capturable.  A cache entry may also set "hh_split" (1-8; default 2
 * below Nk = 256, 4 below Nk = 1024, else 8): the K parts of the hi*hi products of the anti-Hermitian
 * W, V (shorter truncating FP32 chains: accuracy, not speed, so the tuner records
 * it but does not time it).
 * sbe_ctx_tiles: per bucket (ascending Nk) 6 ints (Nk, wires, exchange tile,
 * commutator tile, source tile, hi*hi split) into out (cap ints); *nbuckets = 0
 * before the mixed workspace exists.                                            */
int sbe_autotune(SbeCtx* ctx, const char* cache_json);
int sbe_ctx_tiles(const SbeCtx* ctx, int* out, int cap, int* nbuckets);

/* ---- 1-D PSTD field grid --------------------------------------------------------
 * The reference has no 1-D Maxwell stepper; these entries assemble its pieces:
 * dfdx1D = IFFT(i q FFT f) (PSTD3D/usefulsubs.py:163-185), the grids
 * GetSpaceArray / GetKArray (PSTD3D/typespace.py:815-849, positions;
 * libpulsesuite/helpers.py:838-863, wavenumbers in FFT order), the longitudinal
 * field of ElongfromRho (PSTD3D/rhoPJ.py:703-880, x component) and the mask
 * multiply of ApplyABC (usefulsubs.py:584-609).  Propagation along x (the wire
 * axis); transverse fields E = (Ey, Ez) and H = (Hz, Hy), each 2 x c128 nx;
 * longitudinal Ex (c128 nx).  Leapfrog: H^{n+1/2} = H^{n-1/2} - dt/mu0 curl E^n,
 * E^{n+1} = mask (E^n + dt/eps (curl H^{n+1/2} - J^{n+1/2})), J = (Jy, Jz).      */
typedef struct {
  int nx;              /* grid points: power of two in [256, 65536]            */
  int n_abc;           /* absorbing cells at each end (0: periodic grid)       */
  int pad0, pad1;
  double dx;           /* cell size (m)                                        */
  double epsr;         /* background relative permittivity                     */
  double abc_strength; /* mask = exp(-abc_strength s^2), s = depth in layer    */
} SbePstdDesc;
typedef struct SbePstd SbePstd;
int sbe_pstd_create(const SbePstdDesc* desc, void* stream, SbePstd** out);
int sbe_pstd_destroy(SbePstd* p);
/* device copies of the positions x and wavenumbers q (nx doubles each; NULL skips) */
int sbe_pstd_grid(SbePstd* p, double* x, double* q, void* stream);
/* dfdx1D (usefulsubs.py:163-185) of nf = 1 or 2 fields (nf x c128 nx) into df   */
int sbe_pstd_deriv(SbePstd* p, const double* f, int nf, double* df, void* stream);
int sbe_pstd_update_h(SbePstd* p, const double* E, double* H, double dt, void* stream);
int sbe_pstd_update_e(SbePstd* p, double* E, const double* H, const double* J, double dt,
                      void* stream);
/* update_h then update_e; J may be NULL.  dt must satisfy c dt pi/(sqrt(epsr) dx) <= 2. */
int sbe_pstd_step(SbePstd* p, double* E, double* H, const double* J, double dt, void* stream);
/* Ex from the charge density rho and the polarisation Px (rhoPJ.py:836-866, x only) */
int sbe_pstd_elong(SbePstd* p, const double* rho, const double* Px, double* Ex, void* stream);

/* ---- 3-D PSTD field grid ----------------------------------------------------------
 * Six components on nx x ny x nz (C order, z fastest): E = (Ex, Ey, Ez) and
 * H = (Hx, Hy, Hz), each 3 x c128 N (N = nx ny nz).  The reference has no 3-D
 * Maxwell stepper (its 3-D driver sets E analytically, sbetestpropnov30.py:709); the
 * pieces are the q-space derivative f (i q) along each axis (usefulsubs.py:233-380),
 * the grids (typespace.py:815-849 positions, helpers.py:838-863 FFT-order
 * wavenumbers per axis), the mask multiply of ApplyABC (usefulsubs.py:584-609) and
 * ElongfromRho (rhoPJ.py:703-880).  Leapfrog H^{n+1/2} = H^{n-1/2} - dt/mu0 curl E^n,
 * E^{n+1} = mask (E^n + dt/eps (curl H^{n+1/2} - J)); curl F = IFFT(i q x FFT F).
 * fp32_work: the transforms between the first and last pass in FP32 (the fields
 * stay FP64).                                                                      */
typedef struct {
  int n[3];            /* nx, ny, nz: powers of two in [2, 1024]               */
  int n_abc[3];        /* absorbing cells at both ends of each axis            */
  int fp32_work;       /* 1: FP32 transforms, 0: FP64                          */
  int pad0;
  double d[3];         /* cell sizes (m)                                       */
  double epsr;         /* background relative permittivity                     */
  double abc_strength; /* mask = prod over axes of exp(-abc_strength s^2)      */
} SbePstd3Desc;
typedef struct SbePstd3 SbePstd3;
int sbe_pstd3_create(const SbePstd3Desc* desc, void* stream, SbePstd3** out);
int sbe_pstd3_destroy(SbePstd3* p);
/* device copies of the positions and FFT-order wavenumbers of one axis (NULL skips) */
int sbe_pstd3_grid(SbePstd3* p, int axis, double* x, double* q, void* stream);
/* out = curl F (3 x c128 N each)                                                   */
int sbe_pstd3_curl(SbePstd3* p, const double* F, double* out, void* stream);
int sbe_pstd3_update_h(SbePstd3* p, const double* E, double* H, double dt, void* stream);
int sbe_pstd3_update_e(SbePstd3* p, double* E, const double* H, const double* J, double dt,
                       void* stream);
/* update_h then update_e (J may be NULL); dt <= 2 / (v |q|max) is checked.          */
int sbe_pstd3_step(SbePstd3* p, double* E, double* H, const double* J, double dt, void* stream);
/* rhoPJ.py:703-880 ElongfromRho with the caller's wavenumber tables qx, qy, qz
 * (device, nx / ny / nz doubles; the reference passes its centred GetKxArray...):
 * rho (c128 N), P3 (3 x c128 N) -> out10 = 10 x c128 N [E_PRho x, y, z, E_P x, y, z,
 * E_Rho x, y, z, RhoBound]; P_k (3 x c128 N, may be NULL) receives the transformed P
 * that the reference leaves in its P arguments.  FP64 transforms.                  */
int sbe_pstd3_elong(SbePstd3* p, const double* rho, const double* P3, const double* qx,
                    const double* qy, const double* qz, double* out10, double* P_k,
                    void* stream);

/* ---- wires on the PSTD grid (coupled step) --------------------------------------
 * Field -> wire: Prop2QW (qwoptics.py:667-715) with the grid spline evaluated at
 * x_w + r; wire -> field: QW2Prop (qwoptics.py:717-805, no plasmonic
 * renormalisation) of the real-space sources at x - x_w, summed over wires, and
 * Rho = RhoH - RhoE (SBEs.py:5917).  The soft source is a current sheet at one
 * cell launching E_inc(t) = E0 exp(-((t - tpeak)/tau)^2) cos(w0 (t - tpeak)).  */
typedef struct {
  int src_index;       /* grid cell of the soft source, -1: none               */
  int longitudinal;    /* 1: Ex = longitudinal field of the wires' Rho and Px  */
  int pad0, pad1;
  double E0, tau, w0, tpeak;
  double t0;           /* time of step 0                                       */
} SbeCoupleDesc;
typedef struct SbeCouple SbeCouple;
/* wire_x: HOST array of the nw wire centre positions (m) on the grid.          */
int sbe_couple_create(SbeCtx* ctx, SbePstd* p, const double* wire_x, const SbeCoupleDesc* desc,
                      void* stream, SbeCouple** out);
int sbe_couple_destroy(SbeCouple* cp);
/* Device pointers of the coupling buffers: Ek (per wire 3 x c128 Nr, wire k
 * space), src (per wire 5 x c128 Nr real-space sources), Pg (3 x c128 nx), rho
 * (c128 nx), J (2 x c128 nx).  NULL arguments are skipped.                     */
int sbe_couple_buffers(SbeCouple* cp, double** Ek, double** src, double** Pg, double** rho,
                       double** J);
int sbe_couple_set_step(SbeCouple* cp, long long n, void* stream);
/* Start a new run: step counter 0, previous grid polarisation P^n = 0 (the first
 * current is P^1 / dt, so start the wires from P = 0), Pg, rho and J cleared.  */
int sbe_couple_reset(SbeCouple* cp, void* stream);
/* Sample Ex and E = (Ey, Ez) onto every wire (fills Ek).                       */
int sbe_couple_sample(SbeCouple* cp, const double* Ex, const double* E, void* stream);
/* Deposit the wire sources in src onto the grid (fills Pg and rho).            */
int sbe_couple_deposit(SbeCouple* cp, void* stream);
/* One coupled step t_n -> t_{n+1}: sample E^n, H update, RK4 step of every wire
 * (precision SBE_PREC_FP64 or SBE_PREC_MIXED), deposit, J, E update, Ex.       */
int sbe_couple_step(SbeCouple* cp, double* P, double* C, double* D, double* E, double* H,
                    double* Ex, double dt, int precision, void* stream);
/* CUDA graph of one sbe_couple_step on these buffers (replay with sbe_graph_launch). */
int sbe_couple_graph_create(SbeCouple* cp, double* P, double* C, double* D, double* E, double* H,
                            double* Ex, double dt, int precision, SbeGraph** out,
                            long long* n_kernels);

/* ---- wires along z on the 3-D grid (coupled 3-D step) ------------------------------
 * The reference's 3-D driver (rhoPJ.py:117-488 QuantumWire) samples the grid field on
 * each wire's line (EAtXYZ, usefulsubs.py:1996), steps the wires, forms J = dP/dt and
 * deposits the wire sources with transverse SHO gates exp(-d^2 / (2 a^2))
 * (rhoPJ.py:383-389, QWPlacement :655-702); its wires all share one line along x and
 * it never feeds J back into E.  Here wire w lies along the grid's z axis at
 * (wire_xy[2w], wire_xy[2w + 1]), centred at z = 0, and each wire deposits its own
 * gated sources: the wire's (x, y, z) components are the grid's (z, x, y).  The
 * coupled step feeds J back: sample E^n on every wire (bilinear in x, y, Forsythe-
 * Malcolm-Moler spline along z, window, FFTG as Prop2QW), H update, RK4 of every wire,
 * deposit, J = (P^{n+1} - P^n)/dt plus the soft source (a current sheet in the plane
 * x = x[src_index] along component pol with the profile exp(-(y^2 + z^2)/waist^2)
 * launching E_inc(t) = E0 exp(-((t - tpeak)/tau)^2) cos(w0 (t - tpeak))), E update.  */
typedef struct {
  int src_index;     /* x index of the source plane, -1: none                   */
  int pol;           /* source current component (0 x, 1 y, 2 z)                */
  int pad0, pad1;
  double E0, tau, w0, tpeak;
  double t0;         /* time of step 0                                          */
  double waist;      /* beam waist in the source plane (m); <= 0: plane wave    */
  double gate;       /* transverse gate length a of the deposit (m)             */
} SbeCouple3Desc;
typedef struct SbeCouple3 SbeCouple3;
/* wire_xy: HOST array of 2 nw positions (m) inside the grid's x, y range.          */
int sbe_couple3_create(SbeCtx* ctx, SbePstd3* p, const double* wire_xy, const SbeCouple3Desc* desc,
                       void* stream, SbeCouple3** out);
int sbe_couple3_destroy(SbeCouple3* cp);
/* Device buffers: Ek (per wire 3 x c128 Nr), src (per wire 5 x c128 Nr), J
 * (3 x c128 N), rho (c128 N).  NULL arguments are skipped.                        */
int sbe_couple3_buffers(SbeCouple3* cp, double** Ek, double** src, double** J, double** rho);
/* New run: step 0, previous grid polarisation, J and rho cleared.                   */
int sbe_couple3_reset(SbeCouple3* cp, void* stream);
/* E (3 x c128 N) onto every wire (fills Ek; precision selects the FFTG arithmetic).  */
int sbe_couple3_sample(SbeCouple3* cp, const double* E, int precision, void* stream);
/* The wire sources in src onto the grid: J (with the source at the current step) and rho. */
int sbe_couple3_deposit(SbeCouple3* cp, double dt, void* stream);
int sbe_couple3_step(SbeCouple3* cp, double* P, double* C, double* D, double* E, double* H,
                     double dt, int precision, void* stream);
int sbe_couple3_graph_create(SbeCouple3* cp, double* P, double* C, double* D, double* E,
                             double* H, double dt, int precision, SbeGraph** out,
                             long long* n_kernels);

/* ---- kernel timing (no counterpart in the reference) ------------------------ */
/* enable != 0: record CUDA events around the engine launches of category
 * 0 commutator GEMMs, 1 exchange GEMMs, 2 source GEMMs, 3 FP32 dephasing sums.
 * sbe_ctx_profile_read synchronises, returns total ms and launch count of a
 * category and clears it.                                                      */
int sbe_ctx_profile(SbeCtx* ctx, int enable);
int sbe_ctx_profile_read(SbeCtx* ctx, int category, double* total_ms, long long* launches);

/* ---- carrier-number balance (the FP64 conservation check) ------------------- */
/* The charge normalisation of every step (SBEs.py:5692-5702: ne, nh scaled to
 * their common mean) records, per wire, the carrier numbers it found:
 * out[2w] = sum_k |C_kk|, out[2w + 1] = sum_k |D_kk| after the relaxation and
 * before the normalisation of the last step (FP64; zeros before the first step).
 * |out[2w] - out[2w+1]| / mean is the electron-hole imbalance that step produced.
 * out: host or device memory, 2 * n_wires doubles; waits for the stream.       */
int sbe_ctx_charge(SbeCtx* ctx, double* out, void* stream);

/* ---- device-side error flags (no counterpart in the reference) ------------- */
/* Waits for the stream, then reports whether a bounded wait of the tensor-core
 * engine gave up since the last check (SBE_ERR_TIMEOUT; the flags are cleared). */
int sbe_ctx_check(SbeCtx* ctx, void* stream);
/* Self-test of that path: one launch waits, with the engine's bounded wait, on a
 * barrier nothing completes; the wait gives up after ~2 s and raises the flag that
 * the next sbe_ctx_check reports.  *gave_up = 1 when it did.  Needs the context's
 * mixed-precision workspace (any mixed call creates it); waits for the stream.  */
int sbe_wait_selftest(SbeCtx* ctx, int* gave_up, void* stream);

/* ---- diagnostics ------------------------------------------------------------ */
/* Diagnostic entry, no counterpart in the reference: out[b] = op(A[b]) op(B[b])
 * for a batch of Nk x Nk matrices through the tcgen05 split-precision engine
 * (op: 0 N, 1 T, 2 conj, 3 conj-transpose).  complex_mode 0 uses the real parts
 * only (out imaginary parts are 0).  Nk must be a multiple of 8.               */
int sbe_tc_selftest(int nk, int nbatch, const double* A, const double* B, int opA, int opB,
                    int complex_mode, double* out, void* stream);
/* Diagnostic entry, no counterpart in the reference: the integer-pipe FP64 ->
 * FP32 (round to nearest even; results below 2^-126 flush to zero) and exact
 * FP32 -> FP64 conversions the mixed path uses: f_out[i] = fp32(d_in[i]),
 * d_out[i] = fp64(f_in[i]).                                                    */
int sbe_convert_selftest(const double* d_in, const float* f_in, long long n, float* f_out,
                         double* d_out, void* stream);
/* Diagnostic entry, no counterpart in the reference: the off-diagonal dephasing
 * matrices De, Dh [2Nk+1][Nk] per wire (packed like the context's wires) of the
 * occupations of the states C, D, from the FP64 sums (fp32 = 0, the literal
 * reference loops of dephasing.py:227-317) or from the FP32 sums of the
 * mixed-precision path (fp32 = 1).  Needs a context whose wires all have the
 * OffDiagDph flag.                                                              */
int sbe_deph_selftest(SbeCtx* ctx, const double* C, const double* D, int fp32, double* De,
                      double* Dh, void* stream);

/* ---- 3-D field <-> wire coupling pieces (device pointers, c128 interleaved) -- */
/* rhoPJ.py:491-515 CalcJfx: J[0] = 0, J[i] = J[i-1] - ((new_i - prev_i) / dt) dx
 * (c128 n each).                                                                */
int sbe_calc_jfx(long long n, const double* rho_new, const double* rho_prev, double dt,
                 double dx, double* J, void* stream);
/* rhoPJ.py:655-702 QWPlacement: Fgrid[i][j][k] = gx_i gy_j gz_k Fwire_i (Fgrid c128
 * nx*ny*nz, C order; Fwire c128 nx; gates f64).                                 */
int sbe_qw_placement(int nx, int ny, int nz, const double* Fwire, const double* gx,
                     const double* gy, const double* gz, double* Fgrid, void* stream);
/* usefulsubs.py:1996-2075 EAtXYZ with locator (:1803-1830), batched: out[p] (c128) =
 * trilinear sample of f (c128 nx*ny*nz, C order) on the ascending axes x, y, z at
 * pts[3p..3p+2]; a singleton axis takes its one plane.                         */
int sbe_e_at_xyz(const double* f, const double* x, int nx, const double* y, int ny,
                 const double* z, int nz, const double* pts, int npts, double* out,
                 void* stream);

/* ---- backup files of the state (host only, no device call) ---------------- */
/* Text of SBEs.py:5524-5546 write_sbes_data (WriteSBEsData :6046): one line
 * "re im\n" per complex element, each number as Python's repr of a float64
 * (f"{np.real(val)} {np.imag(val)}").  values: count c128 in host memory, in the
 * file's order (per wire, k2 outer, k1 inner); out needs 50 bytes per value;
 * *written = bytes produced.  threads <= 0: all host threads.                  */
int sbe_backup_format(const double* values, long long count, char* out, long long cap,
                      long long* written, int threads);
/* SBEs.py:5548-5569 read_sbes_data (ReadSBEsData :6051): the first count lines of
 * text, two numbers each (Python float() spellings; further tokens on a line
 * ignored), into values (count c128).  SBE_ERR_ARG on fewer lines or a line that
 * does not start with two numbers.                                              */
int sbe_backup_parse(const char* text, long long len, double* values, long long count,
                     int threads);

#ifdef __cplusplus
}
#endif
#endif /* SBE_GB300_H */
