/*
 * parm_gb300 — C ABI of the GB300 MD time-step library.
 *
 * This is the boundary a host binding (C++, ctypes, SWIG, cgo, ...) links
 * against: plain pointers and sizes, integer status codes, no C++ or CUDA
 * types.  Every function returns PARM_OK (0) or a negative status; the text of
 * the last error of the calling thread is available from parm_last_error().
 *
 * One handle (parm_system) owns the GPU state of `nsys` independent periodic
 * systems (a single simulation is nsys == 1).  Atoms are addressed by their
 * global index: system s owns indices [off_s, off_s + natoms[s]) with off_s the
 * sum of the earlier systems' sizes.  Each entry point names the reference
 * interface (wackywendell/parm, src/...) whose behaviour it provides.
 *
 * Threading: a handle is used from one host thread at a time; all GPU work of
 * a handle runs on the handle's own CUDA stream.
 */
#ifndef PARM_GB300_H
#define PARM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference raises the matching C++ exceptions) */
#define PARM_OK 0
#define PARM_ERR_ARG (-1)      /* std::invalid_argument */
#define PARM_ERR_RUNTIME (-2)  /* std::runtime_error */
#define PARM_ERR_CUDA (-3)     /* CUDA failure (no device, out of memory, ...) */
#define PARM_ERR_CAPACITY (-4) /* neighbour list capacity exceeded; state after the call is invalid */

/* arithmetic of the pair kernels */
#define PARM_FP64 0  /* bit-exact with the reference CPU code */
#define PARM_MIXED 1 /* FP32 pair forces, FP64 integration and reductions */

/* pair interactions (the NListed<A,P> instantiations) */
#define PARM_LJCUT 0     /* NListed<EpsSigCutAtom, LennardJonesCutPair>; params (epsilon, sigma, sigcut) */
#define PARM_REPULSION 1 /* NListed<EpsSigExpAtom, RepulsionPair>;      params (eps, sigma, exponent) */
#define PARM_LJREPULSE 2 /* NListed<EpsSigAtom, LJRepulsePair>;         params (epsilon, sigma, unused) */
#define PARM_LJATTRACTCUT 3 /* NListed<EpsSigCutAtom, LJAttractCutPair> (pyparm's LJAttractCut):
                               LJ attraction only, zero force inside sigma (src/interaction.hpp:154-236,
                               1020-1050); params (epsilon, sigma, sigcut); the mixed path runs it
                               on the per-atom kernels */
/* Kinds 4-17 run on FP64 handles only (a mixed-precision handle rejects
 * them); kinds 4-7 and 9 take four parameters per atom (the atoms' fields). */
#define PARM_LOISOHERN 4     /* NListed<LoisOhernAtom, LoisOhernPair> (sticky spheres, src/interaction.hpp:
                                1679-1744): params (eps, sigma, C, l), C and l averaged */
#define PARM_LOISOHERN_MIN 5 /* NListed<LoisOhernAtom, LoisOhernPairMinCLs> (1746-1751): the smaller C, l */
#define PARM_LOISLIN 6       /* NListed<LoisLinAtom, LoisLinPair> (1764-1829): params (eps, sigma, f, l),
                                the fields LoisLinAtom(eps, sigma, depth, width) stores:
                                f = depth / width (0 for width 0), l = width; f and l averaged */
#define PARM_LOISLIN_MIN 7   /* NListed<LoisLinAtom, LoisLinPairMin> (1831-1836): the smaller f, l */
#define PARM_EISMCLACHLAN 8  /* NListed<EisMclachlanAtom, EisMclachlanPair> (implicit solvation,
                                src/interaction.hpp:1415-1452): params (dist, sigmai, unused);
                                FP64 handles only */
#define PARM_REPULSIONDRAG 9 /* NListed<EpsSigExpDragAtom, RepulsionDragPair> (src/interaction.hpp:
                                1598-1640): soft repulsion minus gamma times the relative normal
                                velocity; params (eps, sigma, exponent, gamma), the fields
                                EpsSigExpDragAtom(eps, sigma, gamma, exponent) stores; FP64 handles
                                only */
/* Indexed epsilons (the IEps*Atom types): the pair's epsilon (and for kinds
 * 10-11 its sigma) comes from the tables of parm_set_pair_table by the two
 * atoms' types, the first atom's row (IEps*Atom::get_epsilon, the first atom
 * being the later one in the neighbour list); params begin with the atom's
 * type index (indx).  FP64 handles only. */
#define PARM_LJCUT_IEPSISIG 10    /* NListed<IEpsISigCutAtom, LennardJonesCutPair> (src/interaction.hpp:
                                     911-954, 977-982): params (indx, sigcut, unused) */
#define PARM_LJATTRACTCUT_IEPSISIG 11 /* NListed<IEpsISigCutAtom, LJAttractCutPair> (1028-1032): same */
#define PARM_LJATTRACTCUT_IEPS 12 /* NListed<IEpsSigCutAtom, LJAttractCutPair> (989-1018, 1033-1037):
                                     params (indx, sigma, sigcut) */
#define PARM_LJATTRACTREPULSE 13  /* NListed<IEpsSigCutAtom, LJAttractRepulsePair> (1251-1298): same */
#define PARM_LJATTRACTFIXEDREPULSE 14 /* NListed<IEpsRepsSigCutAtom, LJAttractFixedRepulsePair>
                                     (1307-1399): params (indx, repeps, sigma, sigcut) */
#define PARM_LJISH 15             /* NListed<IEpsRepsSigExpCutAtom, LJishPair> (1051-1141):
                                     params (indx, repeps, sigma, n, sigcut) */
#define PARM_REPULSION_IEPSISIG 16 /* NListed<IEpsISigExpAtom, RepulsionPair> (pyparm's RepulsionII,
                                     1477-1543): params (indx, exponent, unused) */
#define PARM_LJATTRACTREPULSESIGS 17 /* NListed<EpsEpsSigSigCutAtom, LJAttractRepulseSigsPair>
                                     (1149-1239): params (eps_r, eps_a, sig_r, sig_a, sigcut); FP64
                                     handles only */
/* doubles per atom in parm_set_interaction's params */
#define PARM_NPARAM(kind)                                                                             \
    ((((kind) >= PARM_LOISOHERN && (kind) <= PARM_LOISLIN_MIN) || (kind) == PARM_REPULSIONDRAG ||    \
      (kind) == PARM_LJATTRACTFIXEDREPULSE)                                                           \
         ? 4                                                                                          \
         : (((kind) == PARM_LJISH || (kind) == PARM_LJATTRACTREPULSESIGS) ? 5 : 3))

/* fields of the reference's struct Atom {Vec x, v, a, f; flt m;} (src/box.hpp:234-249) */
#define PARM_X 1u
#define PARM_V 2u
#define PARM_A 4u
#define PARM_F 8u
#define PARM_M 16u

/* parm_evaluate quantities (per system) */
#define PARM_EVAL_ENERGY 0   /* NListed::energy            src/interaction.hpp:2152-2163 */
#define PARM_EVAL_VIRIAL 1   /* NListed::pressure          src/interaction.hpp:2247-2260 */
#define PARM_EVAL_STRESS 2   /* NListed::stress (ndim*ndim) src/interaction.hpp:2278-2291 */
#define PARM_EVAL_CONTACTS 3 /* NListed::contacts          src/interaction.hpp:2124-2137 */
#define PARM_EVAL_OVERLAPS 4 /* NListed::overlaps          src/interaction.hpp:2139-2150 */

/* mean-square-displacement tracker outputs (parm_rsq_get) */
#define PARM_RSQ_XYZ2 0   /* RsqTracker::xyz2   nwin x natoms x ndim  src/constraints.cpp:457-464, 510-518 */
#define PARM_RSQ_XYZ4 1   /* RsqTracker::xyz4   nwin x natoms x ndim  src/constraints.cpp:466-473, 537-545 */
#define PARM_RSQ_R2 2     /* RsqTracker::r2     nwin x natoms         src/constraints.cpp:520-535 */
#define PARM_RSQ_R4 3     /* RsqTracker::r4     nwin x natoms         src/constraints.cpp:475-481, 547-555 */
#define PARM_RSQ_COUNTS 4 /* RsqTracker::counts nwin                  src/constraints.cpp:556-564 */

#define PARM_NOT_MEMBER 0xFFFFFFFFu

typedef struct parm_system parm_system;

/* Text of the calling thread's last error ("" when none). */
const char* parm_last_error(void);

/* Library ABI version (major * 100 + minor). */
int parm_version(void);

/* Select the CUDA device used by handles created afterwards on this thread. */
int parm_use_device(int device);

/* Create a handle for nsys systems of natoms[s] atoms in ndim (2 or 3)
 * dimensions.  Replaces the reference's per-simulation storage:
 * AtomVec(N, mass) (src/box.hpp:441-479) — masses start at 1, all vectors at 0. */
int parm_create(parm_system** out, int ndim, uint32_t nsys, const uint32_t* natoms, int precision);
int parm_destroy(parm_system* s);

/* Box side lengths, nsys*ndim doubles.  OriginBox(Vec size) and
 * OriginBox::resize_to(Vec) without moving atoms (src/box.hpp:97-158, box.cpp:17-20). */
int parm_set_boxes(parm_system* s, const double* L);

/* Copy fields between the handle and host records laid out like the
 * reference's AtomVec storage: record of atom i at atoms + i*stride (stride in
 * doubles, >= 4*ndim+1) holding x[ndim], v[ndim], a[ndim], f[ndim], m.
 * `fields` is an OR of PARM_X..PARM_M.  (AtomVec::operator[], src/box.hpp:470-471) */
int parm_set_atoms(parm_system* s, const double* atoms, uint64_t stride, uint32_t fields);
int parm_get_atoms(parm_system* s, double* atoms, uint64_t stride, uint32_t fields);

/* Install the pair interaction and its neighbour list:
 *   NListed<A,P>(box, atoms, skin) + NListed::add(A) for every atom with
 *   rank[i] != PARM_NOT_MEMBER (src/interaction.hpp:1902-1914).
 * params: natoms*PARM_NPARAM(kind) doubles (see PARM_LJCUT..).  rank[i] is the atom's
 * position in the NeighborList (its insertion order, src/trackers.hpp:194-201),
 * which fixes the reference's pair order; pass NULL for rank[i] = local index.
 * Marks the list for a rebuild on the next update (ignorechanged = true). */
int parm_set_interaction(parm_system* s, int kind, const double* params, const uint32_t* rank,
                         double skin);

/* LeesEdwardsBox (src/box.hpp:165-196, box.cpp:72-135): gamma (nsys values)
 * turns every system's box into a sheared one whose y image shifts x by
 * gamma * Lx (LeesEdwardsBox::diff); NULL returns to OriginBoxes.  FP64
 * handles only; the neighbour lists of a sheared handle are built by an
 * all-pairs test, as the reference's own list build is.  Shearing the atoms
 * (LeesEdwardsBox::shear(dgamma, atoms): x += y dgamma) is the caller's:
 * move them with parm_set_atoms and pass the new gamma here. */
int parm_set_lees_edwards(parm_system* s, const double* gamma);

/* Tables of the indexed kinds (PARM_LJCUT_IEPSISIG ..): eps[a * ntypes + b]
 * is epsilons[b] of the atoms of type a (IEps*Atom::epsilons), sig likewise
 * (IEpsISigCutAtom::sigmas; NULL when no kind in use reads it).  Set before
 * parm_set_interaction with an indexed kind; the next parm_set_interaction
 * applies a change. */
int parm_set_pair_table(parm_system* s, uint32_t ntypes, const double* eps, const double* sig);

/* List diameters given to NeighborList::add(atom, diameter)
 * (src/trackers.hpp:194-201) instead of the pair parameters' max_size():
 * natoms doubles in caller order, NaN where the parameters decide; NULL
 * clears them.  A member with an explicit diameter may have all parameters
 * 0 (added to the list only, as the reference allows: its pairs carry no
 * force).  Takes effect with the next rebuild (ignorechanged = true). */
int parm_set_list_diameters(parm_system* s, const double* diam);

/* NeighborList::ignore(a, b) (src/trackers.hpp:190-193). */
int parm_nlist_ignore(parm_system* s, uint32_t a, uint32_t b);

/* NeighborList::update_list(force) (src/trackers.cpp:19-85).  rebuilt (nsys
 * bytes, may be NULL) receives 1 for systems whose list was rebuilt. */
int parm_nlist_update(parm_system* s, int force, uint8_t* rebuilt);

/* NeighborList::which() and numpairs() per system (src/trackers.hpp:186-187). */
int parm_nlist_which(parm_system* s, uint32_t* which);
int parm_nlist_numpairs(parm_system* s, uint64_t* numpairs);

/* The pair list of system `sys` in the reference's order (NeighborList::begin()
 * .. end(), get(i)): pairs[2k] = first (the later-added atom), pairs[2k+1] =
 * last.  Writes min(cap, npairs) pairs and stores the total in *npairs. */
int parm_nlist_pairs(parm_system* s, uint32_t sys, uint32_t* pairs, uint64_t cap, uint64_t* npairs);

/* Collection::set_forces(constraints_and_a) (src/collection.cpp:159-179). */
int parm_set_forces(parm_system* s, int constraints_and_a);

/* Per-system interaction quantities (PARM_EVAL_*); out holds nsys values
 * (nsys*ndim*ndim for the stress). */
int parm_evaluate(parm_system* s, int what, double* out);

/* Time steps (each equals `nsteps` calls of the reference's timestep()):
 *   CollectionVerlet::timestep  src/collection.cpp:442-469
 *   CollectionDamped::timestep  src/collection.cpp:356-381 (constants 339-354)
 *   CollectionSol::timestep     src/collection.cpp:265-322 (constants 230-263)
 * CollectionSol draws its Gaussian pairs from a counter-based generator
 * (Philox4x32-10 keyed by splitmix64(seed + s), counter = (atom, step)), not
 * from the reference's global Mersenne twister. */
int parm_verlet(parm_system* s, double dt, uint32_t nsteps);
int parm_damped(parm_system* s, double dt, double damping, uint32_t nsteps);
int parm_sol(parm_system* s, double dt, double damping, double T, uint64_t seed, uint32_t nsteps);

/* Conjugate-gradient minimisers, every system with its own line search:
 *   boxed != 0: CollectionNLCG (src/collection.hpp:400-475, src/collection.cpp:494-829),
 *     positions and the box's log-volume, H = U + P0 V; the boxes change
 *     (parm_get_boxes reads them);
 *   boxed == 0: CollectionNLCGV (src/collection.hpp:490-566, src/collection.cpp:877-1168),
 *     positions only.
 * params: nsys x PARM_NLCG_NPARAM doubles in the order of PARM_NLCG_P_*;
 * state (parm_nlcg_get_state / parm_nlcg_set_state): nsys x PARM_NLCG_NSTATE
 * doubles in the order of PARM_NLCG_S_* (the reference's public members).
 * parm_nlcg_init starts every system with all state variables 0 (the
 * constructors); parm_nlcg_set_params changes parameters only (set_max_alpha,
 * set_max_dx, ... and P0, dt, kappa without the reset the reference's setters
 * add: call parm_nlcg_reset for that).  The directions live in the atoms' v
 * and a fields, as in the reference.  Mixed-precision handles switch to the
 * per-atom gather kernel (parm_set_threads_per_atom(101)).  Sums over atoms
 * and pairs are parallel: the scalars agree with the reference to rounding. */
#define PARM_NLCG_NPARAM 11
#define PARM_NLCG_P_DT 0
#define PARM_NLCG_P_P0 1
#define PARM_NLCG_P_KAPPA 2
#define PARM_NLCG_P_KMAX 3
#define PARM_NLCG_P_SECMAX 4
#define PARM_NLCG_P_SECEPS 5
#define PARM_NLCG_P_ALPHAMAX 6
#define PARM_NLCG_P_AFRAC 7
#define PARM_NLCG_P_DXMAX 8
#define PARM_NLCG_P_STEPMAX 9
#define PARM_NLCG_P_MAXDV 10
#define PARM_NLCG_NSTATE 11
#define PARM_NLCG_S_KNEW 0
#define PARM_NLCG_S_K 1
#define PARM_NLCG_S_VL 2
#define PARM_NLCG_S_FL 3
#define PARM_NLCG_S_AL 4
#define PARM_NLCG_S_ALPHA 5
#define PARM_NLCG_S_BETA 6
#define PARM_NLCG_S_BETAUSED 7
#define PARM_NLCG_S_DXSUM 8
#define PARM_NLCG_S_ALPHAVMAX 9
#define PARM_NLCG_S_SEC 10
int parm_nlcg_init(parm_system* s, int boxed, const double* params);
int parm_nlcg_set_params(parm_system* s, const double* params);
int parm_nlcg_get_state(parm_system* s, double* state);
int parm_nlcg_set_state(parm_system* s, const double* state);
/* CollectionNLCG::set_forces(constraints_and_a, true) (collection.cpp:534-566);
 * for CollectionNLCGV, Collection::set_forces (collection.cpp:159-179). */
int parm_nlcg_set_forces(parm_system* s, int constraints_and_a);
/* reset() (collection.cpp:525-532, 977-988), descend() (811-829, 990-1005),
 * `nsteps` calls of timestep() (682-809, 1019-1168). */
int parm_nlcg_reset(parm_system* s);
int parm_nlcg_descend(parm_system* s);
int parm_nlcg_timestep(parm_system* s, uint32_t nsteps);
/* Current box side lengths, nsys*ndim doubles (OriginBox::box_shape, src/box.hpp:114). */
int parm_get_boxes(parm_system* s, double* L);

/* AtomGroup::kinetic_energy(origin) per system (src/box.cpp:401-411);
 * origin: nsys*ndim doubles or NULL. */
int parm_kinetic_energy(parm_system* s, const double* origin, double* out);
/* AtomGroup::momentum() and mass() per system (src/box.cpp:237-258). */
int parm_momentum(parm_system* s, double* momentum, double* mass);
/* max over mobile atoms of |f|^2, per system (minimisation convergence). */
int parm_max_force_sq(parm_system* s, double* out);

/* Mean-square-displacement tracker on the device, replacing RsqTracker
 * (src/constraints.hpp:318-361, src/constraints.cpp:404-560): windows of
 * skips[j] tracker updates; each window keeps, per atom (caller order), the
 * position at its last update and running sums of squared displacements.
 * Positions are measured from each system's centre of mass when usecom
 * (AtomGroup::com), as is.  parm_rsq_start (re)starts the tracker at the
 * current positions (RsqTracker constructor / reset); parm_rsq_update is one
 * RsqTracker::update; while a tracker is running every time step of
 * parm_verlet / parm_damped / parm_sol updates it at the end of the step
 * (Collection::timestep calls update_trackers there), inside the step's
 * CUDA graph.  parm_rsq_get writes the means (PARM_RSQ_*); a window that has
 * not been updated yet divides by a zero count, as the reference does. */
int parm_rsq_start(parm_system* s, const uint64_t* skips, uint32_t nwin, int usecom);
int parm_rsq_update(parm_system* s);
int parm_rsq_get(parm_system* s, int what, double* out);
int parm_rsq_stop(parm_system* s);

/* Freeze systems of a batch: time steps and force evaluations skip the
 * systems whose active[s] is 0 (their atoms, forces and neighbour lists stay
 * as they are; a rebuild test that was due waits until they are stepped
 * again).  All systems start active.  No counterpart in the reference, which
 * runs one system per Collection: this lets a batched minimisation stop the
 * systems that have converged. */
int parm_set_active(parm_system* s, const uint8_t* active);

/* Langevin step counter (advanced once per parm_sol step; the counter used
 * by a step is the value after the advance). */
int parm_get_step(parm_system* s, uint64_t* step);
int parm_set_step(parm_system* s, uint64_t step);

/* Neighbour capacity per atom (grown automatically at set-up from the density). */
int parm_set_nlist_capacity(parm_system* s, uint32_t maxnb);
int parm_get_nlist_capacity(parm_system* s, uint32_t* maxnb);

/* Variant of the mixed-precision pair kernel and list build:
 *   200      cell blocks: the neighbourhood of a block of cells is staged in
 *            shared memory (16-byte records) and the lists hold 16-bit local
 *            indices (default wherever every system has >= 3 cells per axis);
 *   1, 2, 4  threads per atom with neighbour positions staged per tile of 64 atoms;
 *   100 + t  plain gather kernel with t = 1, 4, 8, 16 or 32 threads per atom.
 * Switching converts the current lists (same pairs, same order).  The FP64
 * path always uses one thread per atom, so that each atom's force is summed
 * in the reference's order. */
int parm_set_threads_per_atom(parm_system* s, uint32_t tpa);
/* The variant in use, in the codes of parm_set_threads_per_atom. */
int parm_get_threads_per_atom(parm_system* s, uint32_t* tpa);

/* Time every variant of the mixed-precision pair kernel on the current
 * configuration and keep the fastest; *tpa (when not NULL) receives 2000 for
 * the cell-block kernel, else tiled * 1000 + threads_per_atom * 10 +
 * neighbours_per_iteration.  The state is left unchanged. */
int parm_autotune(parm_system* s, uint32_t* tpa);

/* Cells of the list builds no narrower than `scale` (1 .. 16, default 1)
 * times the largest list radius: wider cells scan more candidates per atom
 * in a rebuild and, for the cell-block kernels, change the blocks.  Results
 * do not depend on it; the lists are rebuilt at the next update. */
int parm_set_cell_scale(parm_system* s, double scale);

/* Steps captured per CUDA graph launch (default 16; 0 launches kernels directly). */
int parm_set_graph_steps(parm_system* s, uint32_t k);

/* Kernel timing: when enabled, time-step calls record CUDA events around the
 * pair-force kernel of every step and accumulate their durations. */
int parm_timing(parm_system* s, int enable);
int parm_timing_read(parm_system* s, double* force_ms, uint64_t* force_launches, double* drift_ms,
                     uint64_t* rebuilds);

/* Number of kernel launches issued by the last time-step call. */
int parm_last_launches(parm_system* s, uint64_t* launches);

/* Wait for all GPU work of the handle. */
int parm_sync(parm_system* s);
/* The handle's cudaStream_t, as an opaque pointer. */
void* parm_stream(parm_system* s);

/* Page-locked host memory for fast parm_set_atoms / parm_get_atoms. */
int parm_host_alloc(void** p, uint64_t bytes);
int parm_host_free(void* p);

/* AtomGroup::kinetic_energy of Atom records that the caller already holds in
 * device memory (stride doubles per record, as for parm_set_atoms), without
 * allocating anything: for callers that cannot allocate device memory
 * (frameworks whose pool owns every device buffer, loops that must not enter
 * the driver's allocator, processes under a fixed device-memory budget).  No
 * counterpart in the reference.  `atoms` and `out` (one double) are device
 * pointers, `origin` a host pointer to ndim doubles or NULL, `stream` a
 * cudaStream_t of the current device (NULL: the legacy default stream; a
 * stream of another device is rejected with PARM_ERR_ARG).  The call is
 * asynchronous on `stream`.
 * At most 262144 atoms per call: the per-atom scratch is a static 2 MiB
 * device array that every GPU loading the library holds until exit.  The
 * first call on a device looks up that array's address, so make it before
 * any stream capture.  All calls share the array: calls that overlap on the
 * GPU race with each other. */
int parm_kinetic_energy_noalloc(const double* atoms, uint64_t stride, uint32_t natoms, int ndim,
                                const double* origin, double* out, void* stream);

/* Evaluate the library's minimum-image routine remainder(d[i], L[i]) on the
 * GPU (test hook for the exact IEEE remainder used by OriginBox::diff). */
int parm_debug_remainder(const double* d, const double* L, double* out, uint32_t n);

/* Test hooks of the Langevin generator.  parm_debug_philox runs the
 * library's Philox4x32-10 block function (Salmon et al., SC'11) on n inputs
 * of 6 words each (counter c0..c3, key k0, k1) and writes 4 words per input.
 * parm_debug_normals writes the 6 standard normals (natoms x 6 doubles) that
 * parm_sol draws for atoms 0..natoms-1 of system `sys` at step counter `step`
 * when called with `seed` (the noise of CollectionSol::timestep,
 * src/collection.cpp:276-283, BivariateGauss::gen_vecs, src/vecrand.cpp:73-85). */
int parm_debug_philox(const uint32_t* in, uint32_t* out, uint32_t n);
int parm_debug_normals(uint64_t seed, uint32_t sys, uint64_t step, uint32_t natoms, double* out);

/* Test hook: the per-atom update's float <-> double conversions on bit
 * patterns, on the GPU: d2f[i] = (float)d[i], f2d[i] = (double)f[i]. */
int parm_debug_fpbits(const double* d, const float* f, uint32_t n, float* d2f, double* f2d);

/* Test hook: atoms staged in shared memory per cell block (the rest of a
 * block's neighbourhood is read from global memory); 0 restores the size
 * chosen from the density.  Results do not depend on it. */
int parm_debug_stage_cap(parm_system* s, uint32_t cap);

#ifdef __cplusplus
}
#endif
#endif
