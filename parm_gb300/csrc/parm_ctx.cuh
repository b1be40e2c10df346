// Device-side context (plain struct of device pointers, passed by value to
// kernels) and the host-callable launchers each translation unit provides.
#pragma once
#include "parm_internal.cuh"

namespace parm {

// integrator / evaluation modes of the pair-force kernels (the epilogue that
// runs once an atom's force is complete)
enum ForceMode : int {
    FM_FORCES = 0,     // Collection::set_forces(false) and time steps: write f
    FM_FORCES_A = 1,   // Collection::set_forces(true):  write f, a = f/m
};

enum DriftMode : int { DM_VERLET = 0, DM_DAMPED = 1, DM_SOL = 2 };

// scalars of the current integrator call, kept in device memory so cached
// graphs do not depend on them (all products formed on the host exactly as
// the reference writes them)
struct StepParams {
    double dt;
    double dt_half;      // dt / 2
    double dt2_half;     // dt * dt / 2
    double c0;           // exp(-damping*dt)
    double c1dt;         // c1 * dt
    double c2dtdt;       // c2 * dt * dt
    double dtc12;        // dt * (c1 - c2)
    double dtc2;         // dt * c2
    double T;            // desired temperature (CollectionSol)
    double x11, x21, x22;// BivariateGauss::set outputs
    int noise;           // damping > 0 in CollectionSol
    int pad;
    unsigned long long step;   // Langevin counter, advanced once per step
};

// Per-system state of the conjugate-gradient minimisers CollectionNLCG /
// CollectionNLCGV (nlcg.cu).  The first 11 doubles are the C ABI's parameter
// vector, the next 11 its state vector (include/parm_gb300.h).
struct NlcgSys {
    double dt, P0, kappa, kmax, secmax, seceps, alphamax, afrac, dxmax, stepmax, maxdV;
    double Knew, k, vl, fl, al, alpha, beta, betaused, dxsum, alphavmax, sec;
    // within a time step
    double eta, eta0, vdv, dx, lfac;
    double iters;   // secant iterations of this time step (a bound on the loop besides sec)
};

struct DevCtx {
    int nd;
    int prec;
    int kind;
    uint32_t nsys;
    uint32_t n;        // total atoms
    uint32_t tpa;      // threads per atom of the mixed-precision pair kernel (1..32)
    uint32_t unr;      // neighbours per thread and iteration in that kernel (1, 2, 4)
    uint32_t tiled;    // use the shared-memory tiled variant (lists via tiles)
    uint32_t maxnb;    // neighbour capacity per atom
    uint32_t uniform;  // UniformFlags
    // every atom has the same pair parameters and list diameter (prm, prm32,
    // diam): a rebuild's permutation leaves those arrays as they are
    uint32_t same_prm;
    // device word: nonzero once an upload gave two atoms different masses;
    // zero, a rebuild's permutation leaves m and invm32 as they are
    uint32_t* m_mixed;
    uint32_t nbucket;  // total buckets (sum over systems of ncell + 1)
    uint32_t any_wrap; // some system has an axis with a single cell (per-pair minimum image)
    uint32_t any_lees; // some system is a LeesEdwardsBox: all-pairs list builds

    const SysConst* sys;
    const uint32_t* bucket_off;   // per system: first bucket (cells, then the non-member bucket)

    // per-atom state (internal order)
    void* x;
    void* v;
    void* a;
    void* f;
    void* lastloc;
    float4* f32;          // mixed-path forces
    double* m;
    float* invm32;        // mixed path: 1/m in FP32 (0 for immobile atoms)
    AtomPrm* prm;
    float4* prm32;        // (sqrt(eps), sigma, third, unused) in FP32; the indexed
                          // kinds keep the atom's type in x (its bit pattern)
    const double* ptab;   // indexed kinds: ptab_n x ptab_n epsilons, then sigmas
    uint32_t ptab_n;
    double* diam;         // A::max_size()
    uint32_t* rank;       // NeighborList position, NOT_MEMBER if not added
    uint32_t* orig;       // caller's atom index (global)
    uint32_t* slot;       // inverse of orig
    uint32_t* atom_sys;   // system of each internal slot (constant)
    uint32_t* nm_rank;    // by orig: rank among the system's non-members
    float4* pos;          // FP32 position view, interleaved per atom:
                          //   pos[2i]   = (coarse X xyz, FP32 list diameter)
                          //   pos[2i+1] = (fine xf xyz, 0)
    uint32_t* bucket;     // current bucket of each internal slot
    float4* posw;         // rebuild only: position relative to its cell's lower corner (FP32), w = list diameter

    // rebuild scratch
    uint32_t* cell_count;
    uint32_t* cell_start;   // start of every bucket; the bucket after a system's cells holds its non-members
    const uint32_t* bucket_sys;  // system of each bucket
    uint32_t* scan_aux;     // per scan block: (segment flag, sum)
    uint32_t* cslot;
    uint32_t* perm;       // new slot -> old slot
    // gather targets for the permutation
    void* x2; void* v2; void* a2; void* f2;
    float4* f32b;
    double* m2; float* invm32b; AtomPrm* prm2; float4* prm32b; double* diam2;
    uint32_t* rank2; uint32_t* orig2; uint32_t* bucket2;

    // neighbour list
    uint32_t* nbr;
    uint32_t* nnb;

    // shared-memory tiles of the mixed-precision pair kernel: TILE_ATOMS
    // consecutive atoms of one system; entries are the tile's distinct
    // (neighbour, periodic image) pairs, the tile lists index them (16 bit)
    uint32_t ntile;
    const uint32_t* tile_atom0;   // first atom of each tile
    const uint32_t* tile_natom;   // atoms in each tile (<= TILE_ATOMS)
    const uint32_t* tile_sys;     // system of each tile
    float4* tile_anchor;          // frame origin (a coarse position, multiple of 1/8)
    uint32_t* tile_ne;            // entries per tile
    unsigned long long* tile_ent; // [t * TILE_ECAP + e]: (neighbour << 12) | image code
    uint16_t* tile_lst;           // [t * maxnb * TILE_ATOMS + k * TILE_ATOMS + a]
    uint32_t* atom_img;           // image of each atom in its tile's frame (4-bit signed per axis)

    // cell-block kernels of the mixed path (staged.cu): blocks of Kx x Ky
    // cells whose neighbourhood is staged in shared memory; 16-bit lists
    uint32_t staged;      // use them (every system has >= 3 cells per axis)
    uint32_t nblk;        // blocks over all systems
    uint32_t stg_cap;     // atoms staged in shared memory per block
    uint32_t stg_prm;     // force kernel: 0 uniform parameters, 1 per-atom sigma, 2 all per atom
    uint32_t stg_dia;     // list build: per-atom list diameters
    const uint4* blk;     // per block: (system, x0 | x1 << 16, y0 | y1 << 16, z)
    float4* stg_tab;      // per block: its table (STG_TAB_WORDS 16-byte words), set by the list build
    uint16_t* nbr16;      // staged lists (layout in staged.cu)
    // per-atom cell-block records (mixed path): see make_record below
    float4* rec;          // cell-block records (fine x, y, z, packed coarse fields), every step
    float4* rframe;       // their frames (fine shift x, y, z, packed coarse offset), each build
    uint32_t* bandn;      // home atoms with a pair in the LJ cut-off band (this force launch)
    uint2* bandq;         // their (block, home index), up to n entries

    // exclusions (NeighborList::ignore), CSR keyed by caller index
    const uint32_t* excl_off;   // n + 1 entries, or null when no exclusions
    const uint32_t* excl_list;

    // per-system control
    const uint32_t* active;  // per system: 0 = frozen (time steps and force launches skip it)
    uint32_t* flag;       // rebuild this step
    uint32_t* force_rb;   // rebuild requested by the host (force / ignorechanged)
    unsigned long long* top;  // [2*s] largest, [2*s+1] second largest squared displacement (bits)
    uint32_t* which;      // NeighborList::which()
    unsigned long long* seed;  // per-system Langevin key
    uint32_t* status;
    uint32_t* any_flag;
    uint32_t* chains;     // rebuild-chain executions (for launch accounting)
    StepParams* params;

    // conjugate-gradient minimisers (nlcg.cu)
    NlcgSys* nlcg;        // per system, or null before parm_nlcg_init
    uint32_t* nlcg_step;  // per system: moves in the current stepx (and is evaluated after it)
    uint32_t* nlcg_loop;  // per system: still in its secant loop
    uint32_t* nlcg_any;   // [0]: some system is still in its secant loop
    uint32_t nlcg_boxed;  // CollectionNLCG (box scaled with kappa) rather than CollectionNLCGV

    // reduction scratch
    // mean-square-displacement tracker (RsqTracker); rsq_n == 0: none
    uint32_t rsq_n;                      // time windows
    uint32_t rsq_com;                    // measure from each system's centre of mass
    const unsigned long long* rsq_skip;  // [rsq_n] window lengths (tracker updates)
    unsigned long long* rsq_cnt;         // [0] tracker time; [1 + j] updates of window j
    double* rsq_past;     // [rsq_n][n][nd] by caller index: position at the window's last update
    double* rsq_x2;       // [rsq_n][n][nd] sums of squared displacements
    double* rsq_x4;       // [rsq_n][n][nd] sums of their squares
    double* rsq_r4;       // [rsq_n][n] sums of squared squared distances
    double* rsq_comv;     // [nsys][3] centre of mass of each system at the current update (or 0)
    double* red;          // per-atom scratch (up to 12 doubles per atom)
    double* sysout;       // per-system outputs
    uint32_t nchunk;      // reduction chunks (up to RED_CHUNK atoms of one system)
    const uint4* chunk;   // (system, first atom, atoms, 0)
    const uint32_t* sys_chunk;   // first chunk of each system (nsys + 1)
    double* part;         // per-chunk partials (up to 12 per chunk)
};

// capi.cu: store the error text returned by parm_last_error(); returns code
int set_error(int code, const char* msg);

// ---- launchers (implemented in the .cu files) ----
// nlist.cu
void launch_arm(const DevCtx& c, cudaStream_t s, int count_step, int use_cond,
                unsigned long long handle);
void launch_rebuild(const DevCtx& c, cudaStream_t s);
void launch_check(const DevCtx& c, cudaStream_t s);
void launch_tiles(const DevCtx& c, cudaStream_t s, int all);   // tiles of every system when all != 0
void launch_numpairs(const DevCtx& c, cudaStream_t s);   // -> sysout[s] (as double)
void launch_posq(const DevCtx& c, cudaStream_t s);
void launch_reframe(const DevCtx& c, cudaStream_t s);
void launch_tables_stg(const DevCtx& c, cudaStream_t s);
// integrate.cu
void launch_drift(const DevCtx& c, cudaStream_t s, int mode, bool with_kick);
void launch_kick(const DevCtx& c, cudaStream_t s, int mode);
void launch_scatter_in(const DevCtx& c, cudaStream_t s, const double* staging, uint64_t stride,
                       uint32_t fields);
void launch_gather_out(const DevCtx& c, cudaStream_t s, double* staging, uint64_t stride,
                       uint32_t fields);
void launch_reduce_atoms(const DevCtx& c, cudaStream_t s, int what, const double* origin);
void launch_rsq(const DevCtx& c, cudaStream_t s, int init);   // tracker start (init) or update
void launch_sys_reduce(const DevCtx& c, cudaStream_t s, int ncomp);
// pair64.cu / pair32.cu
void launch_force64(const DevCtx& c, cudaStream_t s, int mode);
void launch_force32(const DevCtx& c, cudaStream_t s, int mode);
void launch_eval64(const DevCtx& c, cudaStream_t s, int what);
void launch_eval32(const DevCtx& c, cudaStream_t s, int what);
// nlcg.cu (conjugate-gradient minimisers)
enum NlcgPhase : int {
    NP_BEGIN = 0,     // stepx(dt) of a time step
    NP_FL = 1,        // fl from the virial in sysout (boxed)
    NP_ETA0 = 2,      // eta0 = -fdotv; stepx(-dt) next
    NP_LOOPINIT = 3,  // vdv = vdotv; secant loop starts
    NP_PRE = 4,       // secant iteration before its step
    NP_POST = 5,      // secant iteration after its step
    NP_FINISH = 6,    // Polak-Ribiere update of the direction's scalars
    NP_SETF = 7,      // end of set_forces(true, true): al = vl = fl, Knew
    NP_RESET = 8,     // end of reset(): vl = al, k = 0
    NP_DESCEND = 9,   // descend(): al = vl = fl (boxed), stepx(dt) next
};
enum NlcgTerms : int { NT_FV = 0, NT_VV = 1, NT_FA_FF = 2 };
enum NlcgAtoms : int {
    NA_FINISH = 0,    // a = f, v = a + v betaused
    NA_SETF = 1,      // set_forces(true): a = v = f (mobile), 0 otherwise
    NA_RESET = 2,     // reset(): v = a (every atom)
    NA_DESCEND = 3,   // descend(): v = a = f (mobile)
    NA_IMMOBILE_A = 4 // immobile atoms: a = 0 (Collection::set_forces_get_pressure)
};
void launch_nlcg_stepx(const DevCtx& c, cudaStream_t s);
void launch_nlcg_box(const DevCtx& c, cudaStream_t s);
void launch_nlcg_ctl(const DevCtx& c, cudaStream_t s, int phase, int use_cond, unsigned long long handle);
void launch_nlcg_terms(const DevCtx& c, cudaStream_t s, int what, const uint32_t* mask);
void launch_nlcg_atoms(const DevCtx& c, cudaStream_t s, int what);
// staged.cu (mixed path, cell blocks)
void launch_build_stg(const DevCtx& c, cudaStream_t s);
void launch_force_stg(const DevCtx& c, cudaStream_t s, int mode);
void launch_expand_stg(const DevCtx& c, cudaStream_t s);     // staged lists -> nbr (row-major)
void launch_compress_stg(const DevCtx& c, cudaStream_t s);   // nbr (row-major) -> staged lists
int stg_set_smem_limits();   // cudaError_t of raising the kernels' shared-memory limits
// debug entry used by the tests of the minimum-image routine
void launch_remainder_test(const double* d, const double* L, double* out, uint32_t n,
                           cudaStream_t s);
// test hooks of the Langevin generator (integrate.cu)
void launch_philox_test(const uint32_t* in, uint32_t* out, uint32_t n, cudaStream_t s);
void launch_fpbits_test(const double* d, const float* f, uint32_t n, float* d2f, double* f2d, cudaStream_t s);
void launch_normals_test(unsigned long long key, unsigned long long step, uint32_t n, double* out,
                         cudaStream_t s);

// what for launch_eval*: writes per-atom partials into c.red, ncomp per atom
enum EvalWhat : int {
    EV_ENERGY = 0,     // 1 comp
    EV_VIRIAL = 1,     // 1 comp  (sum r.f)
    EV_STRESS = 2,     // nd*nd comps
    EV_CONTACTS = 3,   // 1 comp (count E != 0)
    EV_OVERLAPS = 4,   // 1 comp (count E > 0)
};

// what for launch_reduce_atoms
enum AtomWhat : int {
    AW_KINETIC = 0,    // 1 comp, AtomGroup::kinetic_energy(origin)
    AW_MOMENTUM = 1,   // nd + 1 comps (momentum, mass) over m > 0 finite atoms
    AW_MAXFORCE = 2,   // 1 comp: max |f|^2 over mobile atoms
    AW_COM = 3,        // nd + 1 comps (sum of m x, mass) over m > 0 finite atoms
};

// Cell-block record of an atom (mixed path), 16 bytes, the same for every
// block.  The atom's frame is fixed at each list build: its periodic image m
// (the one nearest to its cell) and, along y and z, the lower edge O of its
// cell row on the 1/8 grid.  With L8 = L rounded to the 1/8 grid:
//   packed coarse fields (units of 1/8, bias 256): x (bits 0-11)
//   8 (X - m L8) + 256, y (bits 12-21) and z (bits 22-31) 8 (X - m L8 - O) + 256;
//   fine part xf - m (L - L8) in FP32,
// so that field / 8 - 32 + fine = x - m L - O.  Atoms stay within the list
// skin of their cell between builds, so the fields stay far from their
// limits; a block moves a record into its own frame with one packed integer
// add per piece (and the fine part of a periodic shift).  The frame itself
// is kept per atom as (fine shift x, y, z, packed coarse offset): packing is
// linear, so the coarse fields are the packed 8 X plus the packed offset.
constexpr int REC_BIAS = 256;

// 8 O: the lower edge of cell row ci (any integer) along axis d on the 1/8 grid
__device__ __forceinline__ int rec_origin8(const SysConst& S, int d, int ci) {
    return (int)floorf(__fmul_rn(__fmul_rn((float)ci, S.cellw32[d]), 8.0f));
}

// the frame of a member atom with position view (A, B) in cell ci; `ok`
// tells whether its fields are in range
template <int ND>
__device__ __forceinline__ float4 rec_frame(const SysConst& S, const uint32_t* ci, const float4& A, const float4& B,
                                            bool& ok) {
    const float X[3] = {A.x, A.y, A.z}, F[3] = {B.x, B.y, B.z};
    int o[3] = {REC_BIAS, REC_BIAS, REC_BIAS};
    float ff[3] = {0.f, 0.f, 0.f};
    ok = true;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        const float cc = __fmul_rn((float)ci[d] + 0.5f, S.cellw32[d]);
        const bool fin = fabsf(X[d]) < 1048576.0f;
        const float m = fin ? rintf(__fmul_rn(__fadd_rn(X[d], F[d]) - cc, S.invLf[d])) : 0.f;
        o[d] = REC_BIAS - (int)m * __float2int_rn(S.L8[d] * 8.0f) - (d == 0 ? 0 : rec_origin8(S, d, (int)ci[d]));
        ff[d] = -m * S.Lr8[d];
        const int g = __float2int_rz(X[d] * 8.0f) + o[d];
        ok = ok && fin && g >= 0 && g < (d == 0 ? 4096 : 1024);
    }
    const uint32_t po = (uint32_t)o[0] + ((uint32_t)o[1] << 12) + ((uint32_t)o[2] << 22);
    return make_float4(ff[0], ff[1], ff[2], __uint_as_float(po));
}

// record from the coarse/fine position view (A, B) and the frame
__device__ __forceinline__ float4 make_record(const float4& A, const float4& B, const float4& fr) {
    const uint32_t w = (uint32_t)__float2int_rz(A.x * 8.0f) + ((uint32_t)__float2int_rz(A.y * 8.0f) << 12) +
                       ((uint32_t)__float2int_rz(A.z * 8.0f) << 22) + __float_as_uint(fr.w);
    return make_float4(B.x + fr.x, B.y + fr.y, B.z + fr.z, __uint_as_float(w));
}

// cell coordinates of local bucket b
__device__ __forceinline__ void cell_coords(const SysConst& S, uint32_t b, uint32_t* ci) {
    ci[0] = b % (uint32_t)S.nc[0];
    ci[1] = (b / (uint32_t)S.nc[0]) % (uint32_t)S.nc[1];
    ci[2] = b / (uint32_t)(S.nc[0] * S.nc[1]);
}

constexpr int BLOCK = 256;
constexpr uint32_t RED_CHUNK = 4096;   // atoms per reduction chunk
constexpr int TILE_ATOMS = 64;
constexpr int TILE_ECAP = 1024;
constexpr int TILE_HASH = 4096;
// cell blocks: at most STG_KY_MAX cell rows along y per block
constexpr int STG_KY_MAX = 6;
constexpr int STG_ROWS_MAX = 3 * (STG_KY_MAX + 2);
constexpr int STG_PIECES_MAX = 3 * STG_ROWS_MAX;
constexpr int STG_KX_MAX = 32;
constexpr int STG_THREADS_HOST = 256;     // threads per block of the cell-block kernels
constexpr uint32_t STG_TAB_WORDS = 160;   // 16-byte words per block table (>= its size)

inline unsigned grid_for(uint32_t n, int block = BLOCK) {
    unsigned g = (unsigned)((n + block - 1) / block);
    return g ? g : 1;
}

}  // namespace parm
