// Host side of the C ABI declared in include/parm_gb300.h: handle
// management, layout conversion, neighbour-list bookkeeping and the
// graph-captured time-step loops.
//
// A time step is captured once per (integrator, steps-per-launch) as a CUDA
// graph:  arm -> IF(rebuild needed) { rebuild chain } -> drift -> pair forces.
// The arm kernel consumes the displacement test accumulated by the previous
// step's force kernel and sets the conditional node's value, so a step without
// a rebuild costs three kernel launches and no host round trip.  The reference
// runs its rebuild test at the end of a step (Collection::update_trackers);
// here it is resolved at the start of the next step, which sees identical
// positions.  Calls that need the reference's post-step list state (queries,
// uploads, force evaluations) first resolve a pending test ("flush").
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "parm_ctx.cuh"
#include "parm_gb300.h"

using namespace parm;

namespace {
thread_local std::string g_err;

// A::max_size() of the atom types (src/interaction.hpp: EpsSigCutAtom 904,
// EpsSigExpAtom 1464, EpsSigAtom 864, LoisOhernAtom 1691, LoisLinAtom 1780,
// EisMclachlanAtom 1423):
// the atom's diameter in its neighbour list
double atom_max_size(int kind, const double* p, const std::vector<double>& tsig, uint32_t ntypes) {
    if (kind == PARM_LJCUT_IEPSISIG || kind == PARM_LJATTRACTCUT_IEPSISIG || kind == PARM_REPULSION_IEPSISIG) {
        // IEpsISigCutAtom::max_size (947-953): the largest sigma of the atom's row times sigcut;
        // IEpsISigExpAtom::max_size (1505-1511): the largest sigma
        const uint32_t t = (uint32_t)p[0];
        if (t >= ntypes || tsig.size() < (size_t)ntypes * ntypes) return 0.0;
        double sg = tsig[(size_t)t * ntypes];
        for (uint32_t k = 1; k < ntypes; ++k)
            if (sg < tsig[(size_t)t * ntypes + k]) sg = tsig[(size_t)t * ntypes + k];
        return kind == PARM_REPULSION_IEPSISIG ? sg : sg * p[1];
    }
    if (kind == PARM_LJATTRACTCUT_IEPS || kind == PARM_LJATTRACTREPULSE) return p[1] * p[2];
    if (kind == PARM_LJATTRACTFIXEDREPULSE) return p[2] * p[3];
    if (kind == PARM_LJISH) return p[2] * p[4];
    if (kind == PARM_LJCUT || kind == PARM_LJATTRACTCUT) return p[1] * p[2];
    if (kind == PARM_LOISOHERN || kind == PARM_LOISOHERN_MIN) return p[1] * (1 + p[2] + p[3]);
    if (kind == PARM_LOISLIN || kind == PARM_LOISLIN_MIN) return p[1] * (1 + p[3]);
    if (kind == PARM_EISMCLACHLAN) return p[0];
    if (kind == PARM_LJATTRACTREPULSESIGS) return p[2] + p[3] * (p[4] - 1);   // EpsEpsSigSigCutAtom (1169)
    return p[1];
}

// device pair law of an API kind (the Lois "Min" variants are a combination flag)
int device_kind(int kind) {
    if (kind == PARM_LOISOHERN || kind == PARM_LOISOHERN_MIN) return KIND_LOISOHERN;
    if (kind == PARM_LOISLIN || kind == PARM_LOISLIN_MIN) return KIND_LOISLIN;
    if (kind == PARM_EISMCLACHLAN) return KIND_EISMCLACHLAN;
    if (kind == PARM_REPULSIONDRAG) return KIND_REPULSIONDRAG;
    if (kind == PARM_LJCUT_IEPSISIG) return KIND_LJCUT_IDX;
    if (kind == PARM_LJATTRACTCUT_IEPSISIG || kind == PARM_LJATTRACTCUT_IEPS) return KIND_LJATTRACT_IDX;
    if (kind == PARM_LJATTRACTREPULSE) return KIND_LJATTRACTREPULSE;
    if (kind == PARM_LJATTRACTFIXEDREPULSE) return KIND_LJFIXEDREPULSE;
    if (kind == PARM_LJISH) return KIND_LJISH;
    if (kind == PARM_REPULSION_IEPSISIG) return KIND_REPULSION_IDX;
    if (kind == PARM_LJATTRACTREPULSESIGS) return KIND_LJATTREPSIGS;
    return kind;
}

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(PARM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define TRY(expr)                 \
    do {                          \
        int r_ = (expr);          \
        if (r_ != PARM_OK) return r_; \
    } while (0)

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct GraphEntry {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaEvent_t> ev;  // per step: drift start, force start, force end
    uint32_t k = 0;
};

enum StepMode { SM_VERLET = 0, SM_DAMPED = 1, SM_SOL = 2, SM_NLCG = 3, SM_NLCGV = 4 };
}  // namespace

namespace parm {
// records an error for parm_last_error() from other translation units
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace parm

struct parm_system {
    DevCtx c{};
    int nd = 3, prec = 0;
    uint32_t nsys = 0, n = 0;
    std::vector<uint32_t> natoms, off;
    std::vector<SysConst> sys;
    std::vector<double> L;
    std::vector<uint32_t> bucket_off;
    int kind = -1;
    double skin = 0.0;
    std::vector<double> prm_in;      // n*3 (global order)
    std::vector<double> ldiam;       // explicit list diameters (global order; NaN: from the parameters), or empty
    uint32_t ntypes = 0;             // indexed kinds: the pair tables (eps then sig, ntypes^2 each)
    std::vector<double> teps, tsig;
    double* ptab_mem = nullptr;
    std::vector<uint32_t> rank_in;   // global order
    std::vector<std::set<uint32_t>> excl;
    bool have_excl = false, excl_dirty = false;
    cudaStream_t st = nullptr, st2 = nullptr;
    std::vector<void*> allocs;
    void* cell_mem = nullptr;
    void* nbr_mem = nullptr;
    void* tlst_mem = nullptr;
    void* excl_mem = nullptr;
    double* staging = nullptr;
    size_t staging_bytes = 0;
    double* d_origin = nullptr;
    StepParams* h_params = nullptr;
    std::map<uint64_t, GraphEntry> graphs;
    uint32_t graph_k = 16;
    bool timing = false;
    double t_force = 0.0, t_drift = 0.0;
    uint64_t n_force = 0, n_rebuild = 0;
    bool pending = false;
    uint64_t last_launches = 0;
    // cell-block kernels of the mixed path (staged.cu)
    void* blk_mem = nullptr;
    void* tab_mem = nullptr;
    void* nbr16_mem = nullptr;
    void* rsq_mem = nullptr;     // mean-square-displacement tracker arrays
    bool want_staged = true;     // prefer them when the grids allow
    bool stg_ok = false;         // the current grids allow them
    bool stg_pending = false;    // grids changed under staged lists: switch back once every system rebuilt
    std::vector<uint32_t> stg_mark;   // which() of each system when the grids changed
    uint32_t stage_cap_override = 0;  // test hook (parm_debug_stage_cap)
    double cell_scale = 1.0;          // cells no narrower than cell_scale x the list radius
    // page-locked words read back on the stream: [0] status, [1] rebuild
    // chains, [2, 2 + nsys) which() before a call, [2 + nsys, 2 + 2 nsys) after
    uint32_t* hst = nullptr;
    // conjugate-gradient minimisers (nlcg.cu): per-system state and flags
    void* nlcg_mem = nullptr;
    bool nlcg_boxed = true;

    ~parm_system() {
        clear_graphs();
        for (void* p : allocs) cudaFree(p);
        if (cell_mem) cudaFree(cell_mem);
        if (nbr_mem) cudaFree(nbr_mem);
        if (tlst_mem) cudaFree(tlst_mem);
        if (blk_mem) cudaFree(blk_mem);
        if (tab_mem) cudaFree(tab_mem);
        if (nbr16_mem) cudaFree(nbr16_mem);
        if (rsq_mem) cudaFree(rsq_mem);
        if (nlcg_mem) cudaFree(nlcg_mem);
        if (ptab_mem) cudaFree(ptab_mem);
        if (excl_mem) cudaFree(excl_mem);
        if (staging) cudaFree(staging);
        if (h_params) cudaFreeHost(h_params);
        if (hst) cudaFreeHost(hst);
        if (st) cudaStreamDestroy(st);
        if (st2) cudaStreamDestroy(st2);
    }

    void clear_graphs() {
        for (auto& kv : graphs) {
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
            if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
            for (cudaEvent_t e : kv.second.ev) cudaEventDestroy(e);
        }
        graphs.clear();
    }

    template <class T>
    int alloc(T*& p, size_t count) {
        void* q = nullptr;
        size_t bytes = std::max<size_t>(count * sizeof(T), 16);
        CUDA_TRY(cudaMalloc(&q, bytes));
        CUDA_TRY(cudaMemsetAsync(q, 0, bytes, st));
        allocs.push_back(q);
        p = static_cast<T*>(q);
        return PARM_OK;
    }
    int allocv(void*& p, size_t count, size_t elem) {
        char* q = nullptr;
        TRY(alloc(q, count * elem));
        p = q;
        return PARM_OK;
    }
    size_t vbytes() const { return nd == 3 ? 32 : 16; }

    // one synchronisation: the status word travels to page-locked host memory
    // on the stream, then the stream is drained
    int sync_status() {
        CUDA_TRY(cudaMemcpyAsync(hst, c.status, 4, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        const uint32_t stw = hst[0];
        if (stw) {
            CUDA_TRY(cudaMemset(c.status, 0, 4));
            if (stw & ST_NBR_OVERFLOW)
                return fail(PARM_ERR_CAPACITY,
                            "neighbour list capacity exceeded (" + std::to_string(c.maxnb) +
                                " per atom); raise it with parm_set_nlist_capacity");
            if (stw & ST_IMAGE_RANGE)
                return fail(PARM_ERR_RUNTIME, "mixed precision: an atom left the coordinate frame of its "
                                              "neighbourhood (positions changed by more than the frame allows "
                                              "without a list rebuild)");
            if (stw & ST_TILE_OVERFLOW)
                return fail(PARM_ERR_CAPACITY, "mixed precision: a tile or cell block has more distinct "
                                               "neighbours than its 16-bit index space (" +
                                                   std::to_string(TILE_ECAP) + " per tile, 65535 per block)");
            if (stw & ST_STAGE_TIMEOUT)
                return fail(PARM_ERR_RUNTIME, "mixed precision: a cell block's shared-memory copies did not "
                                              "complete within the wait limit (forces of the call are invalid)");
            if (stw & ST_SORT_CAP)
                return fail(PARM_ERR_CAPACITY, "FP64 path: a neighbour list exceeded 256 entries");
            if (stw & ST_NONFINITE) return fail(PARM_ERR_RUNTIME, "non-finite atom position");
            return fail(PARM_ERR_RUNTIME, "device status " + std::to_string(stw));
        }
        return PARM_OK;
    }

    // ---- cell grids (depend on the boxes and on the largest list radius) ----
    int setup_cells() {
        double dmax = 0.0;
        bool any_member = false;
        for (uint32_t i = 0; i < n; i++) {
            if (kind < 0 || rank_in[i] == PARM_NOT_MEMBER) continue;
            any_member = true;
            const double* p = &prm_in[(size_t)PARM_NPARAM(kind) * i];
            double d = atom_max_size(kind, p, tsig, ntypes);
            if (!ldiam.empty() && std::isfinite(ldiam[i])) d = ldiam[i];
            dmax = std::max(dmax, d);
        }
        const double rl = dmax + skin;
        std::vector<int> oldnc;
        for (uint32_t s = 0; s < nsys; s++)
            for (int d = 0; d < 3; d++) oldnc.push_back(sys[s].nc[d]);
        bucket_off.assign(nsys + 1, 0);
        uint32_t total = 0;
        for (uint32_t s = 0; s < nsys; s++) {
            SysConst& S = sys[s];
            for (int d = 0; d < 3; d++) S.nc[d] = 1;
            if (any_member && rl > 0.0) {
                for (int d = 0; d < nd; d++) {
                    double w = rl * cell_scale * (1.0 + 1e-9);
                    double q = std::floor(S.L[d] / w);
                    int ncd = q >= 3.0 ? (int)std::min(q, 1024.0) : 1;
                    S.nc[d] = ncd;
                }
                // keep the grid no larger than ~2 cells per atom
                double cap = std::max(64.0, 2.0 * natoms[s]);
                while ((double)S.nc[0] * S.nc[1] * S.nc[2] > cap) {
                    int big = 0;
                    for (int d = 1; d < nd; d++)
                        if (S.nc[d] > S.nc[big]) big = d;
                    S.nc[big] = S.nc[big] * 3 / 4;
                    if (S.nc[big] < 3) S.nc[big] = 1;
                }
            }
            S.ncell = (uint32_t)(S.nc[0] * S.nc[1] * S.nc[2]);
            for (int d = 0; d < 3; d++) {
                S.cellw_inv[d] = (float)(S.nc[d] / S.L[d]);
                S.cellw[d] = S.L[d] / S.nc[d];
                S.cellw32[d] = (float)S.cellw[d];
                const double l8 = std::rint(S.L[d] * 8.0) * 0.125;
                S.L8[d] = (float)l8;
                S.Lr8[d] = (float)(S.L[d] - l8);
            }
            S.skin = skin;
            S.rlist_max = rl;
            S.cellmin = rl * cell_scale * (1.0 + 1e-9);
            S.rec_lim2 = (2.0 * skin + 0.5) * (2.0 * skin + 0.5);
            S.cell_off = total;
            bucket_off[s] = total;
            total += S.ncell + 1;
        }
        bucket_off[nsys] = total;
        c.any_wrap = 0;
        for (uint32_t s2 = 0; s2 < nsys; s2++)
            for (int d = 0; d < nd; d++)
                if (sys[s2].nc[d] < 3) c.any_wrap = 1;
        std::vector<int> newnc;
        for (uint32_t s2 = 0; s2 < nsys; s2++)
            for (int d = 0; d < 3; d++) newnc.push_back(sys[s2].nc[d]);
        if (cell_mem && newnc == oldnc) {
            // same grids: the cell arrays (and staged lists) stay valid; the
            // cell-block records move to the new box's frames
            CUDA_TRY(cudaMemcpyAsync(const_cast<SysConst*>(c.sys), sys.data(), sizeof(SysConst) * nsys,
                                     cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            clear_graphs();
            TRY(plan_blocks());
            if (c.staged) {
                launch_reframe(c, st);
                CUDA_TRY(cudaGetLastError());
                TRY(sync_status());
            }
            return PARM_OK;
        }
        if (c.staged) {
            // the staged lists index the old grids: keep them as row-major lists
            // until every system has been rebuilt on the new grids
            launch_expand_stg(c, st);
            CUDA_TRY(cudaGetLastError());
            TRY(sync_status());
            c.staged = 0;
            stg_pending = true;
            stg_mark.assign(nsys, 0);
            CUDA_TRY(cudaMemcpy(stg_mark.data(), c.which, 4 * nsys, cudaMemcpyDeviceToHost));
        }
        if (cell_mem) cudaFree(cell_mem);
        cell_mem = nullptr;
        const size_t nblk = (total + 4095) / 4096 + 1;
        const size_t words = 3 * (size_t)total + 2 + 2 * nblk;
        CUDA_TRY(cudaMalloc(&cell_mem, words * 4));
        CUDA_TRY(cudaMemsetAsync(cell_mem, 0, words * 4, st));
        c.cell_count = static_cast<uint32_t*>(cell_mem);
        c.cell_start = c.cell_count + total + 1;
        uint32_t* bsys = c.cell_start + total + 1;
        c.bucket_sys = bsys;
        c.scan_aux = bsys + total;
        {
            std::vector<uint32_t> hb(total);
            for (uint32_t s2 = 0; s2 < nsys; s2++)
                for (uint32_t b = bucket_off[s2]; b < bucket_off[s2 + 1]; b++) hb[b] = s2;
            CUDA_TRY(cudaMemcpyAsync(bsys, hb.data(), 4 * (size_t)total, cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaStreamSynchronize(st));
        }
        c.nbucket = total;
        CUDA_TRY(cudaMemcpyAsync(const_cast<SysConst*>(c.sys), sys.data(), sizeof(SysConst) * nsys,
                                 cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(const_cast<uint32_t*>(c.bucket_off), bucket_off.data(),
                                 4 * (nsys + 1), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        clear_graphs();
        return plan_blocks();
    }

    // Cell blocks of the mixed path (staged.cu): blocks of Kx x Ky cells of
    // one z layer holding about 180 atoms; usable when every system has at
    // least 3 cells per axis and the packed coarse fields of the cell-block
    // records fit: x (12 bits) spans the box, y and z (10 bits) a block's
    // neighbourhood, each with 32 length units of head room for the list
    // skin.  Sets stg_ok and, when the blocks are not usable, c.staged = 0.
    int plan_blocks() {
        stg_ok = false;
        // the cell-block kernels serve the LJ, repulsion and WCA laws; the
        // attractive LJ runs on the per-atom kernels
        if (prec != PREC_MIXED || kind < 0 || kind == PARM_LJATTRACTCUT) {
            c.staged = 0;
            return PARM_OK;
        }
        std::vector<uint4> bl;
        double worst = 0.0;
        bool ok = true;
        const double margin = 2.0 * skin + 1.0;
        for (uint32_t s = 0; s < nsys && ok; s++) {
            const SysConst& S = sys[s];
            for (int d = 0; d < nd; d++)
                if (S.nc[d] < 3) ok = false;
            if (!ok) break;
            const double a = std::max(1e-3, (double)natoms[s] / S.ncell);
            // about 0.85 home atoms per thread: nearly every block still fits one
            // pass of its threads, and few threads idle in the pair loop
            const int cells = std::max(1, (int)std::lround(0.85 * STG_THREADS_HOST / a));
            const int ky = std::max(1, std::min({(int)std::lround(std::sqrt(cells / 2.0)), STG_KY_MAX, S.nc[1] - 2}));
            const int kx = std::max(1, std::min({(int)std::lround((double)cells / ky), STG_KX_MAX, S.nc[0] - 2}));
            const int nbx = (S.nc[0] + kx - 1) / kx, nby = (S.nc[1] + ky - 1) / ky;
            const double wx = std::ceil((double)S.nc[0] / nbx), wy = std::ceil((double)S.nc[1] / nby);
            // extents in the block frames (length units): staged fields stay
            // in [0, 3840) / [0, 768) (units of 1/8, bias 256 for the margin)
            const double ex = S.L[0] + 2.0 * S.cellw[0] + margin;
            const double ey = (wy + 2.0) * S.cellw[1] + margin;
            const double ez = nd == 3 ? 3.0 * S.cellw[2] + margin : 0.0;
            if (margin >= 30.0 || ex >= 440.0 || ey >= 60.0 || ez >= 60.0) ok = false;
            worst = std::max(worst, a * (wx + 2) * (wy + 2) * (nd == 3 ? 3 : 1));
            const int nzl = nd == 3 ? S.nc[2] : 1;
            for (int z = 0; z < nzl; z++)
                for (int by = 0; by < nby; by++)
                    for (int bx = 0; bx < nbx; bx++) {
                        const uint32_t x0 = (uint32_t)(bx * S.nc[0] / nbx), x1 = (uint32_t)((bx + 1) * S.nc[0] / nbx);
                        const uint32_t y0 = (uint32_t)(by * S.nc[1] / nby), y1 = (uint32_t)((by + 1) * S.nc[1] / nby);
                        bl.push_back(make_uint4(s, x0 | (x1 << 16), y0 | (y1 << 16), (uint32_t)z));
                    }
        }
        if (!ok || worst > 20000.0 || bl.empty()) {
            c.staged = 0;
            return PARM_OK;
        }
        if (blk_mem) cudaFree(blk_mem);
        blk_mem = nullptr;
        if (tab_mem) cudaFree(tab_mem);
        tab_mem = nullptr;
        CUDA_TRY(cudaMalloc(&blk_mem, sizeof(uint4) * bl.size()));
        CUDA_TRY(cudaMemcpy(blk_mem, bl.data(), sizeof(uint4) * bl.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMalloc(&tab_mem, (size_t)16 * STG_TAB_WORDS * bl.size()));
        c.blk = static_cast<const uint4*>(blk_mem);
        c.stg_tab = static_cast<float4*>(tab_mem);
        c.nblk = (uint32_t)bl.size();
        c.stg_cap = (uint32_t)std::min(4096.0, std::ceil((1.5 * worst + 64.0) / 32.0) * 32.0);
        if (stage_cap_override) c.stg_cap = stage_cap_override;
        const bool uni_eps = c.uniform & UNI_EPS, uni_sig = c.uniform & UNI_SIG, uni_th = c.uniform & UNI_THIRD;
        c.stg_prm = (uni_eps && uni_sig && uni_th) ? 0u : ((uni_eps && uni_th) ? 1u : 2u);
        c.stg_dia = (uni_sig && (kind != PARM_LJCUT || uni_th)) ? 0u : 1u;
        static bool limits_set[256] = {};
        int dev = 0;
        CUDA_TRY(cudaGetDevice(&dev));
        if (dev >= 0 && dev < 256 && !limits_set[dev]) {
            const int e = stg_set_smem_limits();
            if (e != 0) return fail(PARM_ERR_CUDA, "raising the shared-memory limit of the cell-block kernels failed");
            limits_set[dev] = true;
        }
        stg_ok = true;
        if (c.staged) {
            // fresh table memory: the tables of the current cells and box
            launch_tables_stg(c, st);
            CUDA_TRY(cudaGetLastError());
        }
        return PARM_OK;
    }

    // back to the cell-block kernels once every system has been rebuilt on
    // the current grids (their row-major lists then convert exactly)
    int maybe_restage() {
        if (!stg_pending || !want_staged || !stg_ok || c.staged) return PARM_OK;
        std::vector<uint32_t> w(nsys);
        // the handle's stream does not order with the legacy stream of cudaMemcpy
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaMemcpy(w.data(), c.which, 4 * nsys, cudaMemcpyDeviceToHost));
        for (uint32_t s = 0; s < nsys; s++)
            if (w[s] == stg_mark[s]) return PARM_OK;
        launch_compress_stg(c, st);
        launch_reframe(c, st);
        CUDA_TRY(cudaGetLastError());
        c.staged = 1;
        stg_pending = false;
        clear_graphs();
        return sync_status();
    }

    // row-major lists for the kernels that read them (evaluation, pair listing)
    int rowmajor() {
        if (!c.staged) return PARM_OK;
        launch_expand_stg(c, st);
        CUDA_TRY(cudaGetLastError());
        return PARM_OK;
    }

    // (re)allocate the neighbour list; the current lists are kept (a larger
    // capacity only appends columns), so no rebuild is implied
    int set_capacity(uint32_t maxnb) {
        maxnb = std::max<uint32_t>(8, (maxnb + 7) / 8 * 8);
        void* fresh = nullptr;
        if (c.staged && nbr_mem) launch_expand_stg(c, st);   // the staged layout depends on maxnb
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaMalloc(&fresh, (size_t)maxnb * n * 4 + 16));
        if (nbr_mem) {
            // rows are maxnb long: re-pitch the current lists into the new rows
            uint32_t keep = std::min(maxnb, c.maxnb);
            CUDA_TRY(cudaMemcpy2D(fresh, (size_t)maxnb * 4, nbr_mem, (size_t)c.maxnb * 4, (size_t)keep * 4, n,
                                  cudaMemcpyDeviceToDevice));
            if (maxnb < c.maxnb) {
                // shrinking: lists longer than the new capacity are rebuilt
                std::vector<uint32_t> ones(nsys, kind >= 0 ? 1u : 0u);
                CUDA_TRY(cudaMemcpy(c.force_rb, ones.data(), 4 * nsys, cudaMemcpyHostToDevice));
            }
            cudaFree(nbr_mem);
        }
        nbr_mem = fresh;
        c.nbr = static_cast<uint32_t*>(nbr_mem);
        if (c.ntile) {
            // tile lists: [tile][k][atom] with maxnb rows of TILE_ATOMS per tile
            void* tfresh = nullptr;
            const size_t tile_new = (size_t)maxnb * TILE_ATOMS * 2;
            CUDA_TRY(cudaMalloc(&tfresh, tile_new * c.ntile + 16));
            if (tlst_mem) {
                const size_t tile_old = (size_t)c.maxnb * TILE_ATOMS * 2;
                CUDA_TRY(cudaMemcpy2D(tfresh, tile_new, tlst_mem, tile_old, std::min(tile_old, tile_new),
                                      c.ntile, cudaMemcpyDeviceToDevice));
                cudaFree(tlst_mem);
            }
            tlst_mem = tfresh;
            c.tile_lst = static_cast<uint16_t*>(tlst_mem);
        }
        c.maxnb = maxnb;
        if (prec == PREC_MIXED) {
            if (nbr16_mem) cudaFree(nbr16_mem);
            nbr16_mem = nullptr;
            CUDA_TRY(cudaMalloc(&nbr16_mem, (size_t)maxnb * n * 2 + 16));
            c.nbr16 = static_cast<uint16_t*>(nbr16_mem);
            if (c.staged) {
                launch_compress_stg(c, st);
                CUDA_TRY(cudaGetLastError());
                TRY(sync_status());
            }
        }
        clear_graphs();
        return PARM_OK;
    }

    int request_rebuild_all() {
        std::vector<uint32_t> ones(nsys, 1u);
        CUDA_TRY(cudaStreamSynchronize(st));   // a pending test on the stream may still read the flags
        CUDA_TRY(cudaMemcpy(c.force_rb, ones.data(), 4 * nsys, cudaMemcpyHostToDevice));
        return PARM_OK;
    }

    uint32_t estimate_capacity(double density_factor = 1.0) const {
        double worst = 8.0;
        for (uint32_t s = 0; s < nsys; s++) {
            const SysConst& S = sys[s];
            double V = S.L[0] * S.L[1] * (nd == 3 ? S.L[2] : 1.0);
            double rho = density_factor * natoms[s] / V;
            double rl = S.rlist_max;
            double vol = (nd == 3) ? 4.18879020478639 * rl * rl * rl : 3.14159265358979 * rl * rl;
            worst = std::max(worst, rho * vol);
        }
        double est = 1.6 * worst + 24.0;
        if (est > 4096.0) est = 4096.0;
        return (uint32_t)std::ceil(est);
    }

    int upload_exclusions() {
        if (!excl_dirty) return PARM_OK;
        excl_dirty = false;
        if (excl_mem) cudaFree(excl_mem);
        excl_mem = nullptr;
        c.excl_off = nullptr;
        c.excl_list = nullptr;
        if (!have_excl) return PARM_OK;
        std::vector<uint32_t> offs(n + 1, 0), lst;
        for (uint32_t i = 0; i < n; i++) {
            offs[i] = (uint32_t)lst.size();
            for (uint32_t j : excl[i]) lst.push_back(j);
        }
        offs[n] = (uint32_t)lst.size();
        CUDA_TRY(cudaMalloc(&excl_mem, 4 * (offs.size() + lst.size() + 1)));
        uint32_t* p = static_cast<uint32_t*>(excl_mem);
        CUDA_TRY(cudaMemcpy(p, offs.data(), 4 * offs.size(), cudaMemcpyHostToDevice));
        if (!lst.empty())
            CUDA_TRY(cudaMemcpy(p + offs.size(), lst.data(), 4 * lst.size(), cudaMemcpyHostToDevice));
        c.excl_off = p;
        c.excl_list = p + offs.size();
        clear_graphs();
        return PARM_OK;
    }

    // resolve the rebuild test left pending by the last time step
    // arm + IF(rebuild chain) as one cached graph (the rebuild test left
    // pending by the last time step)
    int build_flush_graph(GraphEntry& ge) {
        CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaStreamCaptureStatus cs;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
        cudaGraphConditionalHandle h;
        CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
        launch_arm(c, st, 0, 1, (unsigned long long)h);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
        alignas(cudaGraphNodeParams) unsigned char cpbuf[sizeof(cudaGraphNodeParams)];
        std::memset(cpbuf, 0, sizeof(cpbuf));
        cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cpbuf);
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
        CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CUDA_TRY(cudaStreamBeginCaptureToGraph(st2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        launch_rebuild(c, st2);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamEndCapture(st2, &body));
        CUDA_TRY(cudaStreamEndCapture(st, &ge.graph));
        CUDA_TRY(cudaGraphInstantiate(&ge.exec, ge.graph, 0));
        return PARM_OK;
    }

    int flush() {
        TRY(upload_exclusions());
        if (!pending) return PARM_OK;
        pending = false;
        if (graph_k == 0) {
            launch_arm(c, st, 0, 0, 0);
            launch_rebuild(c, st);
        } else {
            const uint64_t key = ~0ull;   // no time-step graph uses this key
            auto it = graphs.find(key);
            if (it == graphs.end()) {
                GraphEntry ge;
                const int r = build_flush_graph(ge);
                if (r != PARM_OK) {
                    cudaStreamCaptureStatus cs;
                    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
                        cudaGraph_t junk;
                        cudaStreamEndCapture(st, &junk);
                        if (junk) cudaGraphDestroy(junk);
                    }
                    return r;
                }
                it = graphs.emplace(key, ge).first;
            }
            CUDA_TRY(cudaGraphLaunch(it->second.exec, st));
        }
        CUDA_TRY(cudaGetLastError());
        // no synchronisation here: the caller's own call ends with one, which
        // reports any error of these kernels
        return stg_pending ? maybe_restage() : PARM_OK;
    }

    int upload_params(const StepParams& p) {
        *h_params = p;
        // the step counter lives on the device; copy everything before it
        CUDA_TRY(cudaMemcpyAsync(c.params, h_params, offsetof(StepParams, step),
                                 cudaMemcpyHostToDevice, st));
        return PARM_OK;
    }

    int build_graph(int mode, uint32_t k, GraphEntry& ge) {
        ge.k = k;
        if (timing) {
            ge.ev.resize(3 * (size_t)k);
            for (auto& e : ge.ev) CUDA_TRY(cudaEventCreate(&e));
        }
        const int dmode = mode == SM_VERLET ? DM_VERLET : (mode == SM_DAMPED ? DM_DAMPED : DM_SOL);
        const int fmode = FM_FORCES;
        CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (uint32_t step = 0; step < k; step++) {
            cudaStreamCaptureStatus cs;
            cudaGraph_t g = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            size_t ndeps = 0;
            CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
            cudaGraphConditionalHandle h;
            CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
            launch_arm(c, st, 1, 1, (unsigned long long)h);
            CUDA_TRY(cudaGetLastError());
            CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
            // the struct's union has members without default constructors:
            // build it in zeroed storage
            alignas(cudaGraphNodeParams) unsigned char cpbuf[sizeof(cudaGraphNodeParams)];
            std::memset(cpbuf, 0, sizeof(cpbuf));
            cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cpbuf);
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
            CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                                         cudaStreamSetCaptureDependencies));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            CUDA_TRY(cudaStreamBeginCaptureToGraph(st2, body, nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeThreadLocal));
            launch_rebuild(c, st2);
            CUDA_TRY(cudaGetLastError());
            CUDA_TRY(cudaStreamEndCapture(st2, &body));
            if (timing) CUDA_TRY(cudaEventRecordWithFlags(ge.ev[3 * step], st, cudaEventRecordExternal));
            launch_drift(c, st, dmode, step > 0);
            if (timing) CUDA_TRY(cudaEventRecordWithFlags(ge.ev[3 * step + 1], st, cudaEventRecordExternal));
            if (prec == PREC_FP64) launch_force64(c, st, fmode);
            else launch_force32(c, st, fmode);
            if (timing) CUDA_TRY(cudaEventRecordWithFlags(ge.ev[3 * step + 2], st, cudaEventRecordExternal));
            launch_rsq(c, st, 0);   // trackers, at the end of the step (positions final)
            CUDA_TRY(cudaGetLastError());
        }
        launch_kick(c, st, dmode);   // second half of the chunk's last step
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamEndCapture(st, &ge.graph));
        CUDA_TRY(cudaGraphInstantiate(&ge.exec, ge.graph, 0));
        return PARM_OK;
    }

    int run_steps(int mode, uint32_t nsteps) {
        TRY(upload_exclusions());
        CUDA_TRY(cudaMemcpyAsync(hst + 2, c.which, 4 * nsys, cudaMemcpyDeviceToHost, st));
        uint32_t done = 0;
        uint64_t launches = 0;
        if (graph_k == 0) {
            // direct launches (no graph): the rebuild chain is always launched
            // and each of its kernels returns at once for unflagged systems
            const int dmode = mode == SM_VERLET ? DM_VERLET : (mode == SM_DAMPED ? DM_DAMPED : DM_SOL);
            const int fmode = FM_FORCES;
            cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
            if (timing)
                for (auto& q : e) CUDA_TRY(cudaEventCreate(&q));
            for (uint32_t k = 0; k < nsteps; k++) {
                launch_arm(c, st, 1, 0, 0);
                launch_rebuild(c, st);
                if (timing) CUDA_TRY(cudaEventRecord(e[0], st));
                launch_drift(c, st, dmode, k > 0);
                if (timing) CUDA_TRY(cudaEventRecord(e[1], st));
                if (prec == PREC_FP64) launch_force64(c, st, fmode);
                else launch_force32(c, st, fmode);
                if (timing) {
                    CUDA_TRY(cudaEventRecord(e[2], st));
                    CUDA_TRY(cudaEventSynchronize(e[2]));
                    float a = 0.f, b = 0.f;
                    CUDA_TRY(cudaEventElapsedTime(&a, e[0], e[1]));
                    CUDA_TRY(cudaEventElapsedTime(&b, e[1], e[2]));
                    t_drift += a;
                    t_force += b;
                    n_force += 1;
                }
                launch_rsq(c, st, 0);
                CUDA_TRY(cudaGetLastError());
            }
            launch_kick(c, st, dmode);
            if (timing)
                for (auto& q : e) cudaEventDestroy(q);
            launches = (uint64_t)nsteps * (step_kernels() + chain_len()) + 1;
            done = nsteps;
        }
        while (done < nsteps) {
            uint32_t k = std::min(graph_k, nsteps - done);
            uint64_t key = ((uint64_t)mode << 40) | ((uint64_t)k << 1) | (timing ? 1u : 0u);
            auto it = graphs.find(key);
            if (it == graphs.end()) {
                GraphEntry ge;
                int r = build_graph(mode, k, ge);
                if (r != PARM_OK) {
                    cudaStreamCaptureStatus cs;
                    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
                        cudaGraph_t junk;
                        cudaStreamEndCapture(st, &junk);
                        if (junk) cudaGraphDestroy(junk);
                    }
                    return r;
                }
                it = graphs.emplace(key, ge).first;
            }
            CUDA_TRY(cudaGraphLaunch(it->second.exec, st));
            launches += step_kernels() * k + 1;
            if (timing) {
                CUDA_TRY(cudaStreamSynchronize(st));
                for (uint32_t q = 0; q < k; q++) {
                    float a = 0.f, b = 0.f;
                    CUDA_TRY(cudaEventElapsedTime(&a, it->second.ev[3 * q], it->second.ev[3 * q + 1]));
                    CUDA_TRY(cudaEventElapsedTime(&b, it->second.ev[3 * q + 1], it->second.ev[3 * q + 2]));
                    t_drift += a;
                    t_force += b;
                }
                n_force += k;
            }
            done += k;
        }
        pending = true;
        CUDA_TRY(cudaMemcpyAsync(hst + 2 + nsys, c.which, 4 * nsys, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(hst + 1, c.chains, 4, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemsetAsync(c.chains, 0, 4, st));
        TRY(sync_status());
        uint64_t rb = 0;
        for (uint32_t s = 0; s < nsys; s++) rb += (uint64_t)(hst[2 + nsys + s] - hst[2 + s]);
        n_rebuild += rb;
        const uint32_t chains = hst[1];
        last_launches = graph_k == 0 ? launches : launches + (uint64_t)chains * chain_len();
        return maybe_restage();
    }

    // ---- conjugate-gradient minimisers (CollectionNLCG / CollectionNLCGV) ----
    // contexts of the minimiser's kernels: the rebuild works on any grid
    // (per-pair minimum image along single-cell axes, as boxes may shrink
    // below three cells), the pair kernels use the per-atom lists; `cs`
    // evaluates only the systems flagged in nlcg_step
    void nlcg_ctx(DevCtx& cb, DevCtx& cs) const {
        cb = c;
        cb.any_wrap = 1;
        cb.staged = 0;
        cs = cb;
        cs.active = c.nlcg_step;
    }

    // Collection::set_forces_get_pressure(false) of the flagged systems
    // (boxed: + the virial and fl); Collection::set_forces(false) for NLCGV
    void nlcg_forces(const DevCtx& cb, const DevCtx& cs, cudaStream_t q) {
        if (prec == PREC_FP64) launch_force64(cs, q, FM_FORCES);
        else launch_force32(cs, q, FM_FORCES);
        if (!nlcg_boxed) return;
        if (prec == PREC_FP64) launch_eval64(cs, q, EV_VIRIAL);
        else launch_eval32(cs, q, EV_VIRIAL);
        launch_sys_reduce(cb, q, 1);
        launch_nlcg_ctl(cb, q, NP_FL, 0, 0);
    }

    // a conditional node (IF or WHILE on handle h) after the captured work
    // of `q`; `emit` fills its body, captured on st2
    template <class F>
    int nlcg_cond_node(cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, F&& emit) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
        alignas(cudaGraphNodeParams) unsigned char cpbuf[sizeof(cudaGraphNodeParams)];
        std::memset(cpbuf, 0, sizeof(cpbuf));
        cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cpbuf);
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = type;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
        CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CUDA_TRY(cudaStreamBeginCaptureToGraph(st2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        emit(st2);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaStreamEndCapture(st2, &body));
        return PARM_OK;
    }

    int nlcg_new_handle(cudaGraphConditionalHandle& h) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
        CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
        return PARM_OK;
    }

    // the displacement test and, where it fires, the rebuild (update_trackers)
    int nlcg_update_trackers(const DevCtx& cb, bool graph) {
        launch_check(cb, st);
        if (!graph) {
            launch_arm(cb, st, 0, 0, 0);
            launch_rebuild(cb, st);
            CUDA_TRY(cudaGetLastError());
            return PARM_OK;
        }
        cudaGraphConditionalHandle h;
        TRY(nlcg_new_handle(h));
        launch_arm(cb, st, 0, 1, (unsigned long long)h);
        CUDA_TRY(cudaGetLastError());
        return nlcg_cond_node(h, cudaGraphCondTypeIf, [&](cudaStream_t q) { launch_rebuild(cb, q); });
    }

    // one secant iteration (collection.cpp:716-790, 1075-1131) on stream q
    void nlcg_secant(const DevCtx& cb, const DevCtx& cs, cudaStream_t q, int use_cond, unsigned long long h) {
        launch_nlcg_terms(cb, q, NT_FV, c.nlcg_loop);
        launch_sys_reduce(cb, q, 1);
        launch_nlcg_ctl(cb, q, NP_PRE, 0, 0);
        launch_nlcg_stepx(cb, q);
        launch_nlcg_box(cb, q);
        if (!nlcg_boxed) {
            // CollectionNLCGV updates its trackers after every secant step
            launch_check(cb, q);
            launch_arm(cb, q, 0, 0, 0);
            launch_rebuild(cb, q);
        }
        nlcg_forces(cb, cs, q);
        launch_nlcg_ctl(cb, q, NP_POST, use_cond, h);
    }

    // CollectionNLCG::timestep / CollectionNLCGV::timestep for every active system
    int nlcg_emit_step(bool graph, uint32_t max_sec) {
        DevCtx cb, cs;
        nlcg_ctx(cb, cs);
        launch_nlcg_ctl(cb, st, NP_BEGIN, 0, 0);
        launch_nlcg_stepx(cb, st);
        launch_nlcg_box(cb, st);
        nlcg_forces(cb, cs, st);
        launch_nlcg_terms(cb, st, NT_FV, c.nlcg_step);
        launch_sys_reduce(cb, st, 1);
        launch_nlcg_ctl(cb, st, NP_ETA0, 0, 0);
        launch_nlcg_stepx(cb, st);
        launch_nlcg_box(cb, st);
        TRY(nlcg_update_trackers(cb, graph));
        nlcg_forces(cb, cs, st);
        launch_nlcg_terms(cb, st, NT_VV, c.nlcg_step);
        launch_sys_reduce(cb, st, 1);
        CUDA_TRY(cudaGetLastError());
        if (graph) {
            cudaGraphConditionalHandle h;
            TRY(nlcg_new_handle(h));
            launch_nlcg_ctl(cb, st, NP_LOOPINIT, 1, (unsigned long long)h);
            CUDA_TRY(cudaGetLastError());
            TRY(nlcg_cond_node(h, cudaGraphCondTypeWhile,
                               [&](cudaStream_t q) { nlcg_secant(cb, cs, q, 1, (unsigned long long)h); }));
        } else {
            launch_nlcg_ctl(cb, st, NP_LOOPINIT, 0, 0);
            for (uint32_t it = 0; it <= 2 * max_sec + 2; it++) {
                CUDA_TRY(cudaMemcpyAsync(hst, c.nlcg_any, 4, cudaMemcpyDeviceToHost, st));
                CUDA_TRY(cudaStreamSynchronize(st));
                if (!hst[0]) break;
                nlcg_secant(cb, cs, st, 0, 0);
                CUDA_TRY(cudaGetLastError());
            }
        }
        launch_nlcg_terms(cb, st, NT_FA_FF, c.active);
        launch_sys_reduce(cb, st, 2);
        launch_nlcg_ctl(cb, st, NP_FINISH, 0, 0);
        launch_nlcg_atoms(cb, st, NA_FINISH);
        CUDA_TRY(cudaGetLastError());
        return PARM_OK;
    }

    // the boxes after minimiser calls (the device rescales them)
    int nlcg_sync_boxes() {
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaMemcpy(sys.data(), c.sys, sizeof(SysConst) * nsys, cudaMemcpyDeviceToHost));
        c.any_wrap = 0;
        for (uint32_t s = 0; s < nsys; s++)
            for (int d = 0; d < nd; d++) {
                L[(size_t)s * nd + d] = sys[s].L[d];
                if (sys[s].nc[d] < 3) c.any_wrap = 1;
            }
        return PARM_OK;
    }

    // before a minimiser call: pending tests resolved, list capacity for a
    // denser box than the current one (minimisation compresses)
    int nlcg_prepare() {
        if (!c.nlcg) return fail(PARM_ERR_RUNTIME, "parm_nlcg_init has not been called on this handle");
        if (kind < 0) return fail(PARM_ERR_RUNTIME, "no interaction installed");
        TRY(flush());
        uint32_t need = estimate_capacity(1.5);
        if (need > c.maxnb) TRY(set_capacity(need));
        return PARM_OK;
    }

    int nlcg_run(uint32_t nsteps) {
        TRY(nlcg_prepare());
        std::vector<double> hp((size_t)nsys * (sizeof(NlcgSys) / 8));
        uint32_t max_sec = 0;
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaMemcpy(hp.data(), c.nlcg, sizeof(NlcgSys) * nsys, cudaMemcpyDeviceToHost));
        for (uint32_t s = 0; s < nsys; s++)
            max_sec = std::max(max_sec, (uint32_t)std::min(1e6, hp[(size_t)s * (sizeof(NlcgSys) / 8) + 4]));
        uint64_t launches = 0;
        const int mode = nlcg_boxed ? SM_NLCG : SM_NLCGV;
        if (graph_k == 0) {
            for (uint32_t k = 0; k < nsteps; k++) TRY(nlcg_emit_step(false, max_sec));
        } else {
            uint32_t done = 0;
            while (done < nsteps) {
                const uint32_t k = std::min(graph_k, nsteps - done);
                const uint64_t key = ((uint64_t)mode << 40) | ((uint64_t)k << 1);
                auto it = graphs.find(key);
                if (it == graphs.end()) {
                    GraphEntry ge;
                    ge.k = k;
                    int r = PARM_OK;
                    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
                    if (e != cudaSuccess) return fail(PARM_ERR_CUDA, cudaGetErrorString(e));
                    for (uint32_t q = 0; q < k && r == PARM_OK; q++) r = nlcg_emit_step(true, max_sec);
                    cudaGraph_t g = nullptr;
                    e = cudaStreamEndCapture(st, &g);
                    if (r != PARM_OK) {
                        if (g) cudaGraphDestroy(g);
                        return r;
                    }
                    if (e != cudaSuccess) return fail(PARM_ERR_CUDA, cudaGetErrorString(e));
                    ge.graph = g;
                    e = cudaGraphInstantiate(&ge.exec, ge.graph, 0);
                    if (e != cudaSuccess) {
                        cudaGraphDestroy(g);
                        return fail(PARM_ERR_CUDA, cudaGetErrorString(e));
                    }
                    it = graphs.emplace(key, ge).first;
                }
                CUDA_TRY(cudaGraphLaunch(it->second.exec, st));
                launches += 1;
                done += k;
            }
        }
        last_launches = launches;
        TRY(sync_status());
        return nlcg_sync_boxes();
    }

    // kernels in one rebuild chain (launch_rebuild)
    // kernels of one time step outside the rebuild chain: arm, kick-drift,
    // forces (+ the cell-block kernel's band pass for the LJ cut-off)
    uint64_t step_kernels() const {
        return 3 + ((c.prec == PREC_MIXED && c.staged && kind == PARM_LJCUT) ? 1 : 0) +
               (c.rsq_n ? (c.rsq_com ? 5 : 2) : 0);
    }
    uint64_t chain_len() const {
        if (c.prec == PREC_FP64) return 11;
        return (!c.staged && c.ntile && c.tiled) ? 11 : 10;
    }

    int reduce_sys(int ncomp, std::vector<double>& out) {
        launch_sys_reduce(c, st, ncomp);
        CUDA_TRY(cudaGetLastError());
        int nc = ncomp < 0 ? 1 : ncomp;
        out.resize((size_t)nsys * nc);
        CUDA_TRY(cudaMemcpyAsync(out.data(), c.sysout, 8 * out.size(), cudaMemcpyDeviceToHost, st));
        return sync_status();
    }

    int ensure_staging(size_t bytes) {
        if (bytes <= staging_bytes) return PARM_OK;
        if (staging) cudaFree(staging);
        staging = nullptr;
        staging_bytes = 0;
        CUDA_TRY(cudaMalloc(&staging, bytes));
        staging_bytes = bytes;
        return PARM_OK;
    }
};

// field span inside an Atom record: [lo, hi) in doubles
static void field_span(uint32_t fields, int nd, uint64_t& lo, uint64_t& hi) {
    lo = 4 * (uint64_t)nd + 1;
    hi = 0;
    const uint64_t offs[5] = {0, (uint64_t)nd, 2 * (uint64_t)nd, 3 * (uint64_t)nd, 4 * (uint64_t)nd};
    const uint64_t lens[5] = {(uint64_t)nd, (uint64_t)nd, (uint64_t)nd, (uint64_t)nd, 1};
    for (int b = 0; b < 5; b++) {
        if (fields & (1u << b)) {
            lo = std::min(lo, offs[b]);
            hi = std::max(hi, offs[b] + lens[b]);
        }
    }
}

extern "C" {

const char* parm_last_error(void) { return g_err.c_str(); }

int parm_version(void) { return 100; }

int parm_use_device(int device) {
    if (device < 0) return fail(PARM_ERR_ARG, "device must be >= 0");
    CUDA_TRY(cudaSetDevice(device));
    return PARM_OK;
}

int parm_create(parm_system** out, int ndim, uint32_t nsys, const uint32_t* natoms, int precision) {
    if (!out) return fail(PARM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (ndim != 2 && ndim != 3) return fail(PARM_ERR_ARG, "ndim must be 2 or 3");
    if (nsys == 0 || !natoms) return fail(PARM_ERR_ARG, "need at least one system");
    if (precision != PARM_FP64 && precision != PARM_MIXED) return fail(PARM_ERR_ARG, "bad precision");
    uint64_t total = 0;
    for (uint32_t s = 0; s < nsys; s++) total += natoms[s];
    if (total == 0) return fail(PARM_ERR_ARG, "no atoms");
    if (total >= (1ull << 31)) return fail(PARM_ERR_ARG, "too many atoms for one handle");
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    parm_system* S = new parm_system();
    S->nd = ndim;
    S->prec = precision;
    S->nsys = nsys;
    S->n = (uint32_t)total;
    S->natoms.assign(natoms, natoms + nsys);
    S->off.resize(nsys);
    uint32_t o = 0;
    for (uint32_t s = 0; s < nsys; s++) {
        S->off[s] = o;
        o += natoms[s];
    }
    auto bail = [&](int r) {
        delete S;
        return r;
    };
    if (cudaStreamCreateWithFlags(&S->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&S->st2, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(PARM_ERR_CUDA, "cudaStreamCreate failed"));
    DevCtx& c = S->c;
    c.nd = ndim;
    c.prec = precision;
    c.kind = -1;
    c.nsys = nsys;
    c.n = S->n;
    c.tpa = 1;
    c.unr = 1;
    const uint32_t n = S->n;
    const size_t vb = S->vbytes();
    int r = PARM_OK;
#define A(expr)          \
    r = (expr);          \
    if (r != PARM_OK) return bail(r);
    A(S->allocv(c.x, n, vb));
    A(S->allocv(c.v, n, vb));
    A(S->allocv(c.a, n, vb));
    A(S->allocv(c.f, n, vb));
    A(S->allocv(c.lastloc, n, vb));
    A(S->allocv(c.x2, n, vb));
    A(S->allocv(c.v2, n, vb));
    A(S->allocv(c.a2, n, vb));
    A(S->allocv(c.f2, n, vb));
    A(S->alloc(c.f32, n));
    A(S->alloc(c.f32b, n));
    A(S->alloc(c.m, n));
    A(S->alloc(c.m2, n));
    A(S->alloc(c.invm32, n));
    A(S->alloc(c.invm32b, n));
    A(S->alloc(c.prm, n));
    A(S->alloc(c.prm2, n));
    A(S->alloc(c.prm32, n));
    A(S->alloc(c.prm32b, n));
    A(S->alloc(c.diam, n));
    A(S->alloc(c.diam2, n));
    A(S->alloc(c.rank, n));
    A(S->alloc(c.rank2, n));
    A(S->alloc(c.orig, n));
    A(S->alloc(c.orig2, n));
    A(S->alloc(c.slot, n));
    A(S->alloc(c.atom_sys, n));
    A(S->alloc(c.nm_rank, n));
    A(S->alloc(c.bucket, n));
    A(S->alloc(c.bucket2, n));
    A(S->alloc(c.cslot, n));
    A(S->alloc(c.perm, n));
    A(S->alloc(c.nnb, n));
    A(S->alloc(c.pos, 2 * (size_t)n));
    A(S->alloc(c.posw, n));
    A(S->alloc(c.red, (size_t)n * 12));
    {
        uint32_t* act = nullptr;
        A(S->alloc(act, nsys));
        std::vector<uint32_t> ones(nsys, 1u);
        cudaStreamSynchronize(S->st);
        if (cudaMemcpy(act, ones.data(), 4 * (size_t)nsys, cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(PARM_ERR_CUDA, "initial upload failed"));
        c.active = act;
    }
    A(S->alloc(c.flag, nsys));
    A(S->alloc(c.force_rb, nsys));
    A(S->alloc(c.top, 2 * (size_t)nsys));
    A(S->alloc(c.which, nsys));
    A(S->alloc(c.seed, nsys));
    A(S->alloc(c.status, 1));
    A(S->alloc(c.m_mixed, 1));
    A(S->alloc(c.any_flag, 1));
    A(S->alloc(c.chains, 1));
    A(S->alloc(c.params, 1));
    A(S->alloc(c.sysout, (size_t)nsys * 16));
    if (precision == PARM_MIXED) {
        A(S->alloc(c.bandn, 1));
        A(S->alloc(c.bandq, n));
        A(S->alloc(c.rec, n));
        A(S->alloc(c.rframe, n));
    }
    {
        // reduction chunks: consecutive atoms of one system, at least one per system
        std::vector<uint4> ch;
        std::vector<uint32_t> sc(nsys + 1);
        for (uint32_t s = 0; s < nsys; s++) {
            sc[s] = (uint32_t)ch.size();
            uint32_t a = 0;
            do {
                const uint32_t cnt = std::min<uint32_t>(RED_CHUNK, natoms[s] - a);
                ch.push_back(make_uint4(s, S->off[s] + a, cnt, 0u));
                a += cnt;
            } while (a < natoms[s]);
        }
        sc[nsys] = (uint32_t)ch.size();
        uint4* dch = nullptr;
        uint32_t* dsc = nullptr;
        A(S->alloc(dch, ch.size()));
        A(S->alloc(dsc, sc.size()));
        A(S->alloc(c.part, ch.size() * 12));
        cudaStreamSynchronize(S->st);
        if (cudaMemcpy(dch, ch.data(), sizeof(uint4) * ch.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dsc, sc.data(), 4 * sc.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(PARM_ERR_CUDA, "reduction chunk upload failed"));
        c.chunk = dch;
        c.sys_chunk = dsc;
        c.nchunk = (uint32_t)ch.size();
    }
    A(S->alloc(S->d_origin, (size_t)nsys * 3));
    {
        SysConst* dsys = nullptr;
        A(S->alloc(dsys, nsys));
        c.sys = dsys;
        uint32_t* bo = nullptr;
        A(S->alloc(bo, nsys + 1));
        c.bucket_off = bo;
    }
#undef A
    if (cudaMallocHost(&S->h_params, sizeof(StepParams)) != cudaSuccess)
        return bail(fail(PARM_ERR_CUDA, "cudaMallocHost failed"));
    std::memset(S->h_params, 0, sizeof(StepParams));
    if (cudaMallocHost(&S->hst, 4 * (2 + 2 * (size_t)nsys)) != cudaSuccess)
        return bail(fail(PARM_ERR_CUDA, "cudaMallocHost failed"));
    std::memset(S->hst, 0, 4 * (2 + 2 * (size_t)nsys));
    // identity order, masses 1, unit boxes
    std::vector<uint32_t> ident(n), sysid(n), nmr(n);
    for (uint32_t s = 0; s < nsys; s++)
        for (uint32_t i = 0; i < natoms[s]; i++) {
            ident[S->off[s] + i] = S->off[s] + i;
            sysid[S->off[s] + i] = s;
            nmr[S->off[s] + i] = i;
        }
    std::vector<double> ones(n, 1.0);
    std::vector<float> onesf(n, 1.0f);
    std::vector<uint32_t> notm(n, PARM_NOT_MEMBER);
    auto up = [&](void* d, const void* h, size_t bytes) {
        return cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    cudaStreamSynchronize(S->st);
    if (!up(c.orig, ident.data(), 4 * (size_t)n) || !up(c.slot, ident.data(), 4 * (size_t)n) ||
        !up(c.atom_sys, sysid.data(), 4 * (size_t)n) || !up(c.nm_rank, nmr.data(), 4 * (size_t)n) ||
        !up(c.m, ones.data(), 8 * (size_t)n) || !up(c.invm32, onesf.data(), 4 * (size_t)n) ||
        !up(c.rank, notm.data(), 4 * (size_t)n))
        return bail(fail(PARM_ERR_CUDA, "initial upload failed"));
    S->prm_in.assign(3 * (size_t)n, 0.0);
    S->rank_in.assign(n, PARM_NOT_MEMBER);
    S->excl.resize(n);
    S->L.assign((size_t)nsys * ndim, 1.0);
    S->sys.resize(nsys);
    for (uint32_t s = 0; s < nsys; s++) {
        SysConst& Y = S->sys[s];
        std::memset(&Y, 0, sizeof(Y));
        for (int d = 0; d < 3; d++) {
            Y.L[d] = 1.0;
            Y.invL[d] = 1.0;
            Y.halfL[d] = 0.5;
            Y.Lhi[d] = 1.0f;
            Y.Llo[d] = 0.0f;
            Y.invLf[d] = 1.0f;
        }
        Y.atom_off = S->off[s];
        Y.natoms = natoms[s];
    }
    if (precision == PARM_MIXED) {
        std::vector<uint32_t> t0, tn, ts;
        for (uint32_t s = 0; s < nsys; s++)
            for (uint32_t a = 0; a < natoms[s]; a += TILE_ATOMS) {
                t0.push_back(S->off[s] + a);
                tn.push_back(std::min<uint32_t>(TILE_ATOMS, natoms[s] - a));
                ts.push_back(s);
            }
        const uint32_t nt = (uint32_t)t0.size();
        uint32_t *d0 = nullptr, *dn = nullptr, *ds = nullptr;
        r = S->alloc(d0, nt);
        if (r == PARM_OK) r = S->alloc(dn, nt);
        if (r == PARM_OK) r = S->alloc(ds, nt);
        if (r == PARM_OK) r = S->alloc(c.tile_anchor, nt);
        if (r == PARM_OK) r = S->alloc(c.tile_ne, nt);
        if (r == PARM_OK) r = S->alloc(c.tile_ent, (size_t)nt * TILE_ECAP);
        if (r == PARM_OK) r = S->alloc(c.atom_img, n);
        if (r != PARM_OK) return bail(r);
        cudaStreamSynchronize(S->st);
        if (!up(d0, t0.data(), 4 * (size_t)nt) || !up(dn, tn.data(), 4 * (size_t)nt) ||
            !up(ds, ts.data(), 4 * (size_t)nt))
            return bail(fail(PARM_ERR_CUDA, "tile upload failed"));
        c.tile_atom0 = d0;
        c.tile_natom = dn;
        c.tile_sys = ds;
        c.ntile = nt;
        c.tiled = 0;
        c.tpa = 1;
    }
    r = S->setup_cells();
    if (r != PARM_OK) return bail(r);
    r = S->set_capacity(32);
    if (r != PARM_OK) return bail(r);
    *out = S;
    return PARM_OK;
}

int parm_destroy(parm_system* s) {
    if (s) {
        cudaStreamSynchronize(s->st);
        delete s;
    }
    return PARM_OK;
}

int parm_set_boxes(parm_system* S, const double* L) {
    if (!S || !L) return fail(PARM_ERR_ARG, "NULL argument");
    TRY(S->flush());
    for (uint32_t s = 0; s < S->nsys; s++) {
        SysConst& Y = S->sys[s];
        for (int d = 0; d < S->nd; d++) {
            double l = L[(size_t)s * S->nd + d];
            if (!(l > 0.0) || !std::isfinite(l)) return fail(PARM_ERR_ARG, "box lengths must be positive");
            Y.L[d] = l;
            Y.invL[d] = 1.0 / l;
            Y.halfL[d] = 0.5 * l;
            Y.Lhi[d] = (float)l;
            Y.Llo[d] = (float)(l - (double)Y.Lhi[d]);
            Y.invLf[d] = (float)(1.0 / l);
            S->L[(size_t)s * S->nd + d] = l;
        }
    }
    TRY(S->setup_cells());
    if (S->kind >= 0) {
        uint32_t need = S->estimate_capacity();
        if (need > S->c.maxnb) TRY(S->set_capacity(need));
    }
    return PARM_OK;
}

int parm_set_atoms(parm_system* S, const double* atoms, uint64_t stride, uint32_t fields) {
    if (!S || !atoms) return fail(PARM_ERR_ARG, "NULL argument");
    if (stride < 4 * (uint64_t)S->nd + 1) return fail(PARM_ERR_ARG, "stride smaller than an Atom record");
    if (fields & ~31u) return fail(PARM_ERR_ARG, "unknown field bits");
    if (!fields) return PARM_OK;
    TRY(S->flush());
    uint64_t lo, hi;
    field_span(fields, S->nd, lo, hi);
    TRY(S->ensure_staging((size_t)S->n * stride * 8));
    if (2 * (hi - lo) >= stride) {
        // one linear copy of the records beats a strided copy of short rows
        CUDA_TRY(cudaMemcpyAsync(S->staging, atoms, (size_t)S->n * stride * 8, cudaMemcpyHostToDevice, S->st));
    } else {
        CUDA_TRY(cudaMemcpy2DAsync(S->staging + lo, stride * 8, atoms + lo, stride * 8, (hi - lo) * 8, S->n,
                                   cudaMemcpyHostToDevice, S->st));
    }
    launch_scatter_in(S->c, S->st, S->staging, stride, fields);
    CUDA_TRY(cudaGetLastError());
    return S->sync_status();
}

int parm_get_atoms(parm_system* S, double* atoms, uint64_t stride, uint32_t fields) {
    if (!S || !atoms) return fail(PARM_ERR_ARG, "NULL argument");
    if (stride < 4 * (uint64_t)S->nd + 1) return fail(PARM_ERR_ARG, "stride smaller than an Atom record");
    if (fields & ~31u) return fail(PARM_ERR_ARG, "unknown field bits");
    if (!fields) return PARM_OK;
    uint64_t lo, hi;
    field_span(fields, S->nd, lo, hi);
    TRY(S->ensure_staging((size_t)S->n * stride * 8));
    uint64_t covered = 0;
    for (int b = 0; b < 5; b++)
        if (fields & (1u << b)) covered += (b == 4) ? 1 : (uint64_t)S->nd;
    const bool linear = 2 * (hi - lo) >= stride;
    const bool whole = covered == stride;   // every double of each record is written
    if (linear && !whole) {
        // keep the caller's other doubles intact: bring the records over first
        CUDA_TRY(cudaMemcpyAsync(S->staging, atoms, (size_t)S->n * stride * 8, cudaMemcpyHostToDevice, S->st));
    } else if (!linear && covered != hi - lo) {
        CUDA_TRY(cudaMemcpy2DAsync(S->staging + lo, stride * 8, atoms + lo, stride * 8, (hi - lo) * 8,
                                   S->n, cudaMemcpyHostToDevice, S->st));
    }
    launch_gather_out(S->c, S->st, S->staging, stride, fields);
    CUDA_TRY(cudaGetLastError());
    if (linear) {
        CUDA_TRY(cudaMemcpyAsync(atoms, S->staging, (size_t)S->n * stride * 8, cudaMemcpyDeviceToHost, S->st));
    } else {
        CUDA_TRY(cudaMemcpy2DAsync(atoms + lo, stride * 8, S->staging + lo, stride * 8, (hi - lo) * 8, S->n,
                                   cudaMemcpyDeviceToHost, S->st));
    }
    return S->sync_status();
}

int parm_set_interaction(parm_system* S, int kind, const double* params, const uint32_t* rank,
                         double skin) {
    if (!S || !params) return fail(PARM_ERR_ARG, "NULL argument");
    if (kind < 0 || kind > PARM_LJATTRACTREPULSESIGS) return fail(PARM_ERR_ARG, "unknown pair kind");
    const bool indexed = kind >= PARM_LJCUT_IEPSISIG && kind <= PARM_REPULSION_IEPSISIG;
    if (indexed && S->ntypes == 0) return fail(PARM_ERR_ARG, "indexed pair kinds need parm_set_pair_table first");
    if (kind >= PARM_LOISOHERN && S->prec == PREC_MIXED)
        return fail(PARM_ERR_ARG,
                    "the Lois-O'Hern, Lois-Lin, Eis-Mclachlan and drag pairs run on FP64 handles only");
    if (!(skin >= 0.0) || !std::isfinite(skin)) return fail(PARM_ERR_ARG, "skin must be >= 0");
    TRY(S->flush());
    CUDA_TRY(cudaStreamSynchronize(S->st));
    const uint32_t n = S->n;
    S->kind = kind;
    S->skin = skin;
    const size_t np = PARM_NPARAM(kind);
    S->prm_in.assign(params, params + np * n);
    S->rank_in.resize(n);
    for (uint32_t s = 0; s < S->nsys; s++) {
        std::set<uint32_t> seen;
        for (uint32_t i = 0; i < S->natoms[s]; i++) {
            uint32_t g = S->off[s] + i;
            uint32_t rk = rank ? rank[g] : i;
            if (rk != PARM_NOT_MEMBER && !seen.insert(rk).second)
                return fail(PARM_ERR_ARG, "duplicate neighbour-list rank in a system");
            S->rank_in[g] = rk;
        }
    }
    // per-atom parameter records in the caller's order
    std::vector<AtomPrm> prm(n);
    std::vector<float4> prm32(n);
    std::vector<double> diam(n);
    std::vector<uint32_t> nmr(n, 0);
    bool first = true;
    double e0 = 0, s0 = 0, t0 = 0, u0 = 0;
    uint32_t uni = UNI_EPS | UNI_SIG | UNI_THIRD | UNI_FOURTH | UNI_SIG_ONE | UNI_DIAM;
    double d0 = 0;
    for (uint32_t s = 0; s < S->nsys; s++) {
        uint32_t nm = 0;
        for (uint32_t i = 0; i < S->natoms[s]; i++) {
            uint32_t g = S->off[s] + i;
            const double* p = &params[np * g];
            AtomPrm a{p[0], p[1], kind == PARM_LJREPULSE ? 0.0 : p[2], np >= 4 ? p[3] : 0.0,
                      (kind == PARM_LJATTRACTREPULSESIGS) ? p[4] : 0.0};
            uint32_t ptype = 0;
            if (indexed) {
                // records (repeps, sigma, sigcut, p3), the type apart
                const bool member = S->rank_in[g] != PARM_NOT_MEMBER;
                if (member && !(p[0] >= 0.0 && p[0] < (double)S->ntypes && p[0] == std::floor(p[0])))
                    return fail(PARM_ERR_ARG, "type index out of range");
                ptype = member ? (uint32_t)p[0] : 0u;
                if (kind == PARM_LJCUT_IEPSISIG || kind == PARM_LJATTRACTCUT_IEPSISIG || kind == PARM_REPULSION_IEPSISIG)
                    a = AtomPrm{0.0, 0.0, p[1], 0.0, 0.0};   // sigcut, or the exponent
                else if (kind == PARM_LJATTRACTCUT_IEPS || kind == PARM_LJATTRACTREPULSE)
                    a = AtomPrm{0.0, p[1], p[2], 0.0, 0.0};
                else if (kind == PARM_LJATTRACTFIXEDREPULSE) a = AtomPrm{p[1], p[2], p[3], 0.0, 0.0};
                else a = AtomPrm{p[1], p[2], p[4], p[3], 0.0};
                if (kind == PARM_LJCUT_IEPSISIG) a.p3 = 1 - 1 / std::pow(a.p2, 6);      // LennardJonesCut ctor
                if (kind == PARM_LJATTRACTREPULSE) a.p3 = 1 - std::pow(a.p2, -6);      // its cut energy term
                if (kind == PARM_LJATTRACTFIXEDREPULSE) a.p3 = 1 - std::pow(a.p2, -6.0);
            }
            if (kind == PARM_LJCUT) a.p3 = 1 - 1 / std::pow(a.p2, 6);  // LennardJonesCut ctor
            if (kind == PARM_LJATTRACTCUT || kind == PARM_LJATTRACTCUT_IEPSISIG || kind == PARM_LJATTRACTCUT_IEPS) {
                // LJAttract::energy(cut) (interaction.hpp:170-177), times epsilon in the pair
                const double rsig = a.p2;
                if (rsig < 1) {
                    a.p3 = -1;
                } else {
                    const double rsq = rsig * rsig;
                    const double rsix = rsq * rsq * rsq;
                    const double mid = (1 - 1 / rsix);
                    a.p3 = mid * mid - 1;
                }
            }
            prm[g] = a;
            prm32[g] = (kind == PARM_EISMCLACHLAN)
                           ? make_float4((float)a.p0, (float)a.p1, 0.f, 0.f)   // (dist, sigmai)
                           : make_float4((float)std::sqrt(a.p0), (float)a.p1, (float)a.p2, (float)a.p3);
            if (indexed) {
                float tf;
                std::memcpy(&tf, &ptype, 4);
                prm32[g].x = tf;   // the type's bit pattern
            }
            diam[g] = atom_max_size(kind, p, S->tsig, S->ntypes);
            const bool explicit_d = !S->ldiam.empty() && std::isfinite(S->ldiam[g]);
            if (explicit_d) diam[g] = S->ldiam[g];   // NeighborList::add(atom, diameter)
            if (S->rank_in[g] == PARM_NOT_MEMBER) {
                nmr[g] = nm++;
                continue;
            }
            if (kind == PARM_EISMCLACHLAN) {
                if (!(a.p0 >= 0.0 && std::isfinite(a.p0) && std::isfinite(a.p1)))
                    return fail(PARM_ERR_ARG, "dist must be finite and >= 0, sigmai finite");
            } else if (kind == PARM_LJATTRACTREPULSESIGS) {
                if (!(a.p0 >= 0.0 && a.p1 >= 0.0 && a.p2 > 0.0 && a.p3 > 0.0 && a.p4 > 0.0 && std::isfinite(a.p4)))
                    return fail(PARM_ERR_ARG, "epsilons must be >= 0, sigmas and sigcut > 0");
            } else if (indexed) {
                const bool sig_ok = (kind <= PARM_LJATTRACTCUT_IEPSISIG || kind == PARM_REPULSION_IEPSISIG) || a.p1 > 0.0;
                if (!(sig_ok && a.p0 >= 0.0 && a.p2 >= 0.0 && std::isfinite(a.p2) && (kind != PARM_LJISH || a.p3 > 0.0)))
                    return fail(PARM_ERR_ARG, "sigma and n must be > 0, repeps and sigcut >= 0");
            } else if (!(a.p0 >= 0.0) || !(a.p1 > 0.0 || (explicit_d && a.p1 == 0.0 && a.p0 == 0.0))) {
                return fail(PARM_ERR_ARG, "sigma must be > 0, epsilon >= 0");
            }
            if (np == 4 && !indexed &&
                !(std::isfinite(a.p2) && std::isfinite(a.p3) && a.p2 >= 0.0 && a.p3 >= 0.0))
                return fail(PARM_ERR_ARG, "the third and fourth parameters must be finite and >= 0");
            if (first) {
                e0 = a.p0;
                s0 = a.p1;
                t0 = a.p2;
                u0 = a.p3;
                d0 = diam[g];
                first = false;
            }
            if (diam[g] != d0) uni &= ~UNI_DIAM;
            if (a.p0 != e0) uni &= ~UNI_EPS;
            if (a.p1 != s0) uni &= ~UNI_SIG;
            if (a.p2 != t0) uni &= ~UNI_THIRD;
            if (a.p3 != u0) uni &= ~UNI_FOURTH;
            if (a.p1 != 1.0) uni &= ~UNI_SIG_ONE;
        }
    }
    // explicit list diameters: no uniform-threshold shortcut in the list builds
    if (!S->ldiam.empty()) uni &= ~UNI_SIG;
    if (!(uni & UNI_SIG)) uni &= ~UNI_SIG_ONE;
    // internal order of the device arrays
    std::vector<uint32_t> orig(n);
    CUDA_TRY(cudaMemcpy(orig.data(), S->c.orig, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    std::vector<AtomPrm> prm_k(n);
    std::vector<float4> prm32_k(n);
    std::vector<double> diam_k(n);
    std::vector<uint32_t> rank_k(n);
    for (uint32_t k = 0; k < n; k++) {
        uint32_t g = orig[k];
        prm_k[k] = prm[g];
        prm32_k[k] = prm32[g];
        diam_k[k] = diam[g];
        rank_k[k] = S->rank_in[g];
    }
    CUDA_TRY(cudaMemcpy(S->c.prm, prm_k.data(), sizeof(AtomPrm) * n, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(S->c.prm32, prm32_k.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(S->c.diam, diam_k.data(), 8 * (size_t)n, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(S->c.rank, rank_k.data(), 4 * (size_t)n, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(S->c.nm_rank, nmr.data(), 4 * (size_t)n, cudaMemcpyHostToDevice));
    bool same = true;
    for (uint32_t k = 1; k < n && same; k++)
        same = std::memcmp(&prm_k[k], &prm_k[0], sizeof(AtomPrm)) == 0 &&
               std::memcmp(&prm32_k[k], &prm32_k[0], sizeof(float4)) == 0 &&
               std::memcmp(&diam_k[k], &diam_k[0], sizeof(double)) == 0;
    S->c.same_prm = same ? 1u : 0u;
    if (kind == PARM_LOISOHERN_MIN || kind == PARM_LOISLIN_MIN) uni |= COMB_MIN;
    if (indexed || kind == PARM_LJATTRACTREPULSESIGS) {
        // per-pair values from the tables, or a fifth parameter: no per-atom shortcuts
        uni &= ~(UNI_EPS | UNI_SIG_ONE);
        if (kind == PARM_LJCUT_IEPSISIG || kind == PARM_LJATTRACTCUT_IEPSISIG || kind == PARM_REPULSION_IEPSISIG)
            uni |= IDX_SIG;
    }
    S->c.kind = device_kind(kind);
    S->c.uniform = uni;
    launch_posq(S->c, S->st);
    CUDA_TRY(cudaGetLastError());
    TRY(S->setup_cells());
    uint32_t need = S->estimate_capacity();
    if (need > S->c.maxnb) TRY(S->set_capacity(need));
    // every list is rebuilt next (ignorechanged), in the preferred format
    const uint32_t was = S->c.staged;
    S->c.staged = (S->stg_ok && S->want_staged) ? 1u : 0u;
    S->stg_pending = false;
    if (S->c.staged != was) S->clear_graphs();
    return S->request_rebuild_all();  // ignorechanged = true
}

int parm_set_lees_edwards(parm_system* S, const double* gamma) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (gamma && S->prec != PREC_FP64) return fail(PARM_ERR_ARG, "Lees-Edwards boxes run on FP64 handles only");
    if (gamma && S->nd < 2) return fail(PARM_ERR_ARG, "Lees-Edwards boxes need two or three dimensions");
    if (gamma)
        for (uint32_t s = 0; s < S->nsys; s++)
            if (!std::isfinite(gamma[s])) return fail(PARM_ERR_ARG, "non-finite shear");
    TRY(S->flush());
    CUDA_TRY(cudaStreamSynchronize(S->st));
    S->c.any_lees = gamma ? 1u : 0u;
    for (uint32_t s = 0; s < S->nsys; s++) {
        S->sys[s].lees = gamma ? 1 : 0;
        S->sys[s].gamma = gamma ? gamma[s] : 0.0;
    }
    CUDA_TRY(cudaMemcpy(const_cast<SysConst*>(S->c.sys), S->sys.data(), sizeof(SysConst) * S->nsys,
                        cudaMemcpyHostToDevice));
    S->clear_graphs();
    return S->kind >= 0 ? S->request_rebuild_all() : PARM_OK;
}

int parm_set_pair_table(parm_system* S, uint32_t ntypes, const double* eps, const double* sig) {
    if (!S || !eps) return fail(PARM_ERR_ARG, "NULL argument");
    if (ntypes == 0 || ntypes > 4096) return fail(PARM_ERR_ARG, "ntypes must be 1 .. 4096");
    const size_t nn = (size_t)ntypes * ntypes;
    for (size_t k = 0; k < nn; k++)
        if (!std::isfinite(eps[k]) || (sig && !std::isfinite(sig[k]))) return fail(PARM_ERR_ARG, "non-finite table entry");
    TRY(S->flush());
    CUDA_TRY(cudaStreamSynchronize(S->st));
    S->ntypes = ntypes;
    S->teps.assign(eps, eps + nn);
    if (sig) S->tsig.assign(sig, sig + nn);
    else S->tsig.assign(nn, 0.0);
    if (S->ptab_mem) cudaFree(S->ptab_mem);
    S->ptab_mem = nullptr;
    CUDA_TRY(cudaMalloc(&S->ptab_mem, 16 * nn));
    CUDA_TRY(cudaMemcpy(S->ptab_mem, S->teps.data(), 8 * nn, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(S->ptab_mem + nn, S->tsig.data(), 8 * nn, cudaMemcpyHostToDevice));
    S->c.ptab = S->ptab_mem;
    S->c.ptab_n = ntypes;
    return PARM_OK;
}

int parm_set_list_diameters(parm_system* S, const double* diam) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (!diam) {
        S->ldiam.clear();
    } else {
        for (uint32_t i = 0; i < S->n; i++)
            if (diam[i] < 0.0 || std::isinf(diam[i])) return fail(PARM_ERR_ARG, "list diameters must be >= 0 or NaN");
        S->ldiam.assign(diam, diam + S->n);
    }
    if (S->kind < 0) return PARM_OK;   // applied by the next parm_set_interaction
    const std::vector<double> prm = S->prm_in;
    const std::vector<uint32_t> rk = S->rank_in;
    return parm_set_interaction(S, S->kind, prm.data(), rk.data(), S->skin);
}

int parm_nlist_ignore(parm_system* S, uint32_t a, uint32_t b) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (a >= S->n || b >= S->n) return fail(PARM_ERR_ARG, "atom index out of range");
    TRY(S->flush());
    S->excl[a].insert(b);
    S->excl[b].insert(a);
    S->have_excl = true;
    S->excl_dirty = true;
    // ignorechanged = true for the system(s) involved
    uint32_t sa = (uint32_t)(std::upper_bound(S->off.begin(), S->off.end(), a) - S->off.begin() - 1);
    uint32_t sb = (uint32_t)(std::upper_bound(S->off.begin(), S->off.end(), b) - S->off.begin() - 1);
    uint32_t one = 1;
    CUDA_TRY(cudaStreamSynchronize(S->st));
    CUDA_TRY(cudaMemcpy(S->c.force_rb + sa, &one, 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(S->c.force_rb + sb, &one, 4, cudaMemcpyHostToDevice));
    return PARM_OK;
}

int parm_nlist_update(parm_system* S, int force, uint8_t* rebuilt) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    TRY(S->flush());
    if (S->kind < 0) {
        if (rebuilt) std::memset(rebuilt, 0, S->nsys);
        return PARM_OK;
    }
    if (force) {
        std::vector<uint32_t> ones(S->nsys, 1u);
        CUDA_TRY(cudaMemcpyAsync(S->c.force_rb, ones.data(), 4 * S->nsys, cudaMemcpyHostToDevice, S->st));
    } else {
        launch_check(S->c, S->st);
    }
    launch_arm(S->c, S->st, 0, 0, 0);
    launch_rebuild(S->c, S->st);
    CUDA_TRY(cudaGetLastError());
    TRY(S->sync_status());
    TRY(S->maybe_restage());
    if (rebuilt) {
        std::vector<uint32_t> fl(S->nsys);
        CUDA_TRY(cudaMemcpy(fl.data(), S->c.flag, 4 * S->nsys, cudaMemcpyDeviceToHost));
        for (uint32_t s = 0; s < S->nsys; s++) rebuilt[s] = fl[s] ? 1 : 0;
    }
    return PARM_OK;
}

int parm_nlist_which(parm_system* S, uint32_t* which) {
    if (!S || !which) return fail(PARM_ERR_ARG, "NULL argument");
    TRY(S->flush());
    CUDA_TRY(cudaStreamSynchronize(S->st));   // the pending test may still run on the handle's stream
    CUDA_TRY(cudaMemcpy(which, S->c.which, 4 * S->nsys, cudaMemcpyDeviceToHost));
    return PARM_OK;
}

int parm_nlist_numpairs(parm_system* S, uint64_t* numpairs) {
    if (!S || !numpairs) return fail(PARM_ERR_ARG, "NULL argument");
    TRY(S->flush());
    TRY(S->rowmajor());
    launch_numpairs(S->c, S->st);
    std::vector<double> out;
    TRY(S->reduce_sys(1, out));
    for (uint32_t s = 0; s < S->nsys; s++) numpairs[s] = (uint64_t)(out[s] + 0.5);
    return PARM_OK;
}

int parm_nlist_pairs(parm_system* S, uint32_t sys, uint32_t* pairs, uint64_t cap, uint64_t* npairs) {
    if (!S || !npairs) return fail(PARM_ERR_ARG, "NULL argument");
    if (sys >= S->nsys) return fail(PARM_ERR_ARG, "system index out of range");
    TRY(S->flush());
    TRY(S->rowmajor());
    CUDA_TRY(cudaStreamSynchronize(S->st));   // lists of a pending rebuild, complete
    const uint32_t o = S->off[sys], na = S->natoms[sys], mx = S->c.maxnb;
    std::vector<uint32_t> nnb(na), rank(S->n), orig(na), nbr((size_t)na * mx);
    CUDA_TRY(cudaMemcpy(nnb.data(), S->c.nnb + o, 4 * (size_t)na, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(rank.data(), S->c.rank, 4 * (size_t)S->n, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(orig.data(), S->c.orig + o, 4 * (size_t)na, cudaMemcpyDeviceToHost));
    if (na && mx)
        CUDA_TRY(cudaMemcpy(nbr.data(), S->c.nbr + (size_t)o * mx, 4 * (size_t)na * mx, cudaMemcpyDeviceToHost));
    struct P {
        uint32_t r1, r2, a, b;
    };
    std::vector<P> v;
    for (uint32_t i = 0; i < na; i++) {
        uint32_t ri = rank[o + i];
        if (ri == PARM_NOT_MEMBER) continue;
        for (uint32_t k = 0; k < nnb[i]; k++) {
            uint32_t j = nbr[(size_t)i * mx + k];
            uint32_t rj = rank[j];
            if (rj < ri) v.push_back({ri, rj, orig[i], orig[j - o]});
        }
    }
    std::sort(v.begin(), v.end(), [](const P& x, const P& y) {
        return x.r1 != y.r1 ? x.r1 < y.r1 : x.r2 < y.r2;
    });
    *npairs = v.size();
    if (pairs) {
        uint64_t m = std::min<uint64_t>(cap, v.size());
        for (uint64_t k = 0; k < m; k++) {
            pairs[2 * k] = v[k].a;
            pairs[2 * k + 1] = v[k].b;
        }
    }
    return PARM_OK;
}

int parm_set_forces(parm_system* S, int constraints_and_a) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    TRY(S->flush());
    const int mode = constraints_and_a ? FM_FORCES_A : FM_FORCES;
    if (S->prec == PREC_FP64) launch_force64(S->c, S->st, mode);
    else launch_force32(S->c, S->st, mode);
    CUDA_TRY(cudaGetLastError());
    return S->sync_status();
}

int parm_evaluate(parm_system* S, int what, double* out) {
    if (!S || !out) return fail(PARM_ERR_ARG, "NULL argument");
    if (what < 0 || what > 4) return fail(PARM_ERR_ARG, "unknown quantity");
    TRY(S->flush());
    const int ncomp = what == PARM_EVAL_STRESS ? S->nd * S->nd : 1;
    if (S->kind < 0) {
        std::fill(out, out + (size_t)S->nsys * ncomp, 0.0);
        return PARM_OK;
    }
    if (S->prec == PREC_FP64) launch_eval64(S->c, S->st, what);
    else {
        TRY(S->rowmajor());
        launch_eval32(S->c, S->st, what);
    }
    CUDA_TRY(cudaGetLastError());
    std::vector<double> v;
    TRY(S->reduce_sys(ncomp, v));
    std::copy(v.begin(), v.end(), out);
    return PARM_OK;
}

int parm_verlet(parm_system* S, double dt, uint32_t nsteps) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (nsteps == 0) return PARM_OK;
    StepParams p{};
    p.dt = dt;
    p.dt_half = dt / 2;
    p.dt2_half = dt * dt / 2;
    TRY(S->upload_params(p));
    return S->run_steps(SM_VERLET, nsteps);
}

int parm_damped(parm_system* S, double dt, double damping, uint32_t nsteps) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (!(dt > 0)) return fail(PARM_ERR_ARG, "Collection::CollectionSol: dt >= 0");
    if (nsteps == 0) return PARM_OK;
    // CollectionDamped::set_constants (collection.cpp:339-354)
    double c0, c1, c2;
    if (damping <= 0.0) {
        c0 = 1;
        c1 = 1;
        c2 = .5;
    } else {
        double dampdt = damping * dt;
        c0 = std::exp(-dampdt);
        c1 = (-std::expm1(-dampdt)) / dampdt;
        c2 = (1 - c1) / dampdt;
    }
    StepParams p{};
    p.dt = dt;
    p.c0 = c0;
    p.c1dt = c1 * dt;
    p.c2dtdt = c2 * dt * dt;
    p.dtc12 = dt * (c1 - c2);
    p.dtc2 = dt * c2;
    TRY(S->upload_params(p));
    return S->run_steps(SM_DAMPED, nsteps);
}

int parm_sol(parm_system* S, double dt, double damping, double T, uint64_t seed, uint32_t nsteps) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (!(dt > 0)) return fail(PARM_ERR_ARG, "Collection::CollectionSol: dt >= 0");
    if (nsteps == 0) return PARM_OK;
    // CollectionSol::set_constants (collection.cpp:230-263) and BivariateGauss::set (vecrand.cpp:48-62)
    double c0, c1, c2, sigmar, sigmav, corr;
    const double force_mag = damping;
    if (force_mag <= 0.0) {
        c0 = 1;
        c1 = 1;
        c2 = .5;
        sigmar = 0;
        sigmav = 0;
        corr = 1;
    } else {
        double dampdt = force_mag * dt;
        c0 = std::exp(-dampdt);
        c1 = (-std::expm1(-dampdt)) / dampdt;
        c2 = (1 - c1) / dampdt;
        if (dampdt > 1e-4)
            sigmar = std::sqrt((1 / dampdt) * (2 - (-4 * std::expm1(-dampdt) + std::expm1(-2 * dampdt)) / dampdt));
        else
            sigmar = std::sqrt(2 * dampdt / 3 - dampdt * dampdt / 2 + 7 * dampdt * dampdt * dampdt / 30);
        sigmav = std::sqrt(-std::expm1(-2 * dampdt));
        double exdpdt = (-std::expm1(-dampdt));
        corr = exdpdt * exdpdt / dampdt / sigmar / sigmav;
    }
    if (!(sigmar >= 0) || !(sigmav >= 0) || !(corr >= 0) || !(corr <= 1))
        return fail(PARM_ERR_ARG, "BivariateGauss::set: invalid constants");
    StepParams p{};
    p.dt = dt;
    p.c0 = c0;
    p.c1dt = c1 * dt;
    p.c2dtdt = c2 * dt * dt;
    p.dtc12 = dt * (c1 - c2);
    p.dtc2 = dt * c2;
    p.T = T;
    p.x11 = sigmar;
    p.x21 = sigmav * corr;
    p.x22 = sigmav * std::sqrt(1 - corr * corr);
    p.noise = damping > 0 ? 1 : 0;
    std::vector<unsigned long long> seeds(S->nsys);
    for (uint32_t s = 0; s < S->nsys; s++) seeds[s] = splitmix64(seed + s);
    CUDA_TRY(cudaMemcpyAsync(S->c.seed, seeds.data(), 8 * S->nsys, cudaMemcpyHostToDevice, S->st));
    TRY(S->upload_params(p));
    return S->run_steps(SM_SOL, nsteps);
}

int parm_kinetic_energy(parm_system* S, const double* origin, double* out) {
    if (!S || !out) return fail(PARM_ERR_ARG, "NULL argument");
    if (origin)
        CUDA_TRY(cudaMemcpyAsync(S->d_origin, origin, 8 * (size_t)S->nsys * S->nd, cudaMemcpyHostToDevice,
                                 S->st));
    launch_reduce_atoms(S->c, S->st, AW_KINETIC, origin ? S->d_origin : nullptr);
    CUDA_TRY(cudaGetLastError());
    std::vector<double> v;
    TRY(S->reduce_sys(1, v));
    std::copy(v.begin(), v.end(), out);
    return PARM_OK;
}

int parm_momentum(parm_system* S, double* momentum, double* mass) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    launch_reduce_atoms(S->c, S->st, AW_MOMENTUM, nullptr);
    CUDA_TRY(cudaGetLastError());
    std::vector<double> v;
    TRY(S->reduce_sys(S->nd + 1, v));
    for (uint32_t s = 0; s < S->nsys; s++) {
        for (int d = 0; d < S->nd; d++)
            if (momentum) momentum[(size_t)s * S->nd + d] = v[(size_t)s * (S->nd + 1) + d];
        if (mass) mass[s] = v[(size_t)s * (S->nd + 1) + S->nd];
    }
    return PARM_OK;
}

// ---- mean-square-displacement tracker (RsqTracker) ----
int parm_rsq_start(parm_system* S, const uint64_t* skips, uint32_t nskip, int usecom) {
    if (!S || !skips) return fail(PARM_ERR_ARG, "NULL argument");
    if (nskip == 0 || nskip > 64) return fail(PARM_ERR_ARG, "1 to 64 time windows");
    for (uint32_t j = 0; j < nskip; j++)
        if (skips[j] == 0) return fail(PARM_ERR_ARG, "window lengths must be >= 1");
    TRY(S->flush());
    CUDA_TRY(cudaStreamSynchronize(S->st));
    if (S->rsq_mem) cudaFree(S->rsq_mem);
    S->rsq_mem = nullptr;
    S->c.rsq_n = 0;
    const size_t per = (size_t)nskip * S->n;
    const size_t bytes = 8 * ((size_t)nskip + 1 + nskip + 3 * per * S->nd + per + 3 * (size_t)S->nsys);
    CUDA_TRY(cudaMalloc(&S->rsq_mem, bytes));
    CUDA_TRY(cudaMemsetAsync(S->rsq_mem, 0, bytes, S->st));
    unsigned long long* skip = static_cast<unsigned long long*>(S->rsq_mem);
    CUDA_TRY(cudaMemcpyAsync(skip, skips, 8 * (size_t)nskip, cudaMemcpyHostToDevice, S->st));
    S->c.rsq_skip = skip;
    S->c.rsq_cnt = skip + nskip;
    double* d = reinterpret_cast<double*>(S->c.rsq_cnt + nskip + 1);
    S->c.rsq_past = d;
    S->c.rsq_x2 = d + per * S->nd;
    S->c.rsq_x4 = d + 2 * per * S->nd;
    S->c.rsq_r4 = d + 3 * per * S->nd;
    S->c.rsq_comv = S->c.rsq_r4 + per;
    S->c.rsq_com = usecom ? 1u : 0u;
    S->c.rsq_n = nskip;
    S->clear_graphs();
    launch_rsq(S->c, S->st, 1);   // the windows start at the current positions
    CUDA_TRY(cudaGetLastError());
    return S->sync_status();
}

int parm_rsq_update(parm_system* S) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (!S->c.rsq_n) return fail(PARM_ERR_ARG, "no tracker (parm_rsq_start)");
    TRY(S->flush());
    launch_rsq(S->c, S->st, 0);
    CUDA_TRY(cudaGetLastError());
    return S->sync_status();
}

int parm_rsq_get(parm_system* S, int what, double* out) {
    if (!S || !out) return fail(PARM_ERR_ARG, "NULL argument");
    const uint32_t nw = S->c.rsq_n;
    if (!nw) return fail(PARM_ERR_ARG, "no tracker (parm_rsq_start)");
    if (what < PARM_RSQ_XYZ2 || what > PARM_RSQ_COUNTS) return fail(PARM_ERR_ARG, "unknown tracker output");
    TRY(S->flush());
    const size_t n = S->n, nd = (size_t)S->nd, per = (size_t)nw * n;
    std::vector<unsigned long long> cnt(nw + 1);
    CUDA_TRY(cudaMemcpyAsync(cnt.data(), S->c.rsq_cnt, 8 * (nw + 1), cudaMemcpyDeviceToHost, S->st));
    std::vector<double> v;
    if (what != PARM_RSQ_COUNTS) {
        const double* src = what == PARM_RSQ_XYZ4 ? S->c.rsq_x4 : (what == PARM_RSQ_R4 ? S->c.rsq_r4 : S->c.rsq_x2);
        v.resize(what == PARM_RSQ_R4 ? per : per * nd);
        CUDA_TRY(cudaMemcpyAsync(v.data(), src, 8 * v.size(), cudaMemcpyDeviceToHost, S->st));
    }
    TRY(S->sync_status());
    // means over each window's updates, as RsqTracker1::xyz2 / xyz4 / r4 and
    // RsqTracker::r2 (the row sum of the xyz2 means)
    for (uint32_t j = 0; j < nw; j++) {
        const double count = (double)cnt[1 + j];
        if (what == PARM_RSQ_COUNTS) {
            out[j] = count;
        } else if (what == PARM_RSQ_R2) {
            for (size_t i = 0; i < n; i++) {
                const double* row = &v[(j * n + i) * nd];
                double sum = row[0] / count;
                for (size_t d = 1; d < nd; d++) sum = sum + row[d] / count;
                out[j * n + i] = sum;
            }
        } else if (what == PARM_RSQ_R4) {
            for (size_t i = 0; i < n; i++) out[j * n + i] = v[j * n + i] / count;
        } else {
            for (size_t k = 0; k < n * nd; k++) out[j * n * nd + k] = v[j * n * nd + k] / count;
        }
    }
    return PARM_OK;
}

int parm_rsq_stop(parm_system* S) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    TRY(S->flush());
    CUDA_TRY(cudaStreamSynchronize(S->st));
    if (S->rsq_mem) cudaFree(S->rsq_mem);
    S->rsq_mem = nullptr;
    S->c.rsq_n = 0;
    S->clear_graphs();
    return PARM_OK;
}

int parm_max_force_sq(parm_system* S, double* out) {
    if (!S || !out) return fail(PARM_ERR_ARG, "NULL argument");
    launch_reduce_atoms(S->c, S->st, AW_MAXFORCE, nullptr);
    CUDA_TRY(cudaGetLastError());
    std::vector<double> v;
    TRY(S->reduce_sys(-1, v));
    std::copy(v.begin(), v.end(), out);
    return PARM_OK;
}

int parm_get_step(parm_system* S, uint64_t* step) {
    if (!S || !step) return fail(PARM_ERR_ARG, "NULL argument");
    CUDA_TRY(cudaStreamSynchronize(S->st));
    CUDA_TRY(cudaMemcpy(step, &S->c.params->step, 8, cudaMemcpyDeviceToHost));
    return PARM_OK;
}

int parm_set_step(parm_system* S, uint64_t step) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    CUDA_TRY(cudaStreamSynchronize(S->st));
    CUDA_TRY(cudaMemcpy(&S->c.params->step, &step, 8, cudaMemcpyHostToDevice));
    return PARM_OK;
}

int parm_set_nlist_capacity(parm_system* S, uint32_t maxnb) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (maxnb == 0 || maxnb > 65536) return fail(PARM_ERR_ARG, "capacity must be in 1..65536");
    TRY(S->flush());
    return S->set_capacity(maxnb);
}

int parm_get_nlist_capacity(parm_system* S, uint32_t* maxnb) {
    if (!S || !maxnb) return fail(PARM_ERR_ARG, "NULL argument");
    *maxnb = S->c.maxnb;
    return PARM_OK;
}

// switch the mixed path between the cell-block kernels and the gather /
// tiled kernels, converting the current lists (same pairs)
static int set_staged(parm_system* S, bool on) {
    if (on == (S->c.staged != 0)) return PARM_OK;
    if (on) {
        if (!S->stg_ok) return fail(PARM_ERR_ARG, "the cell-block kernel needs >= 3 cells per axis in every system");
        if (S->stg_pending) return PARM_OK;   // switches after the next rebuild of every system
        launch_compress_stg(S->c, S->st);
        launch_reframe(S->c, S->st);
        S->c.staged = 1;
    } else {
        launch_expand_stg(S->c, S->st);
        S->c.staged = 0;
    }
    CUDA_TRY(cudaGetLastError());
    S->clear_graphs();
    return S->sync_status();
}

int parm_set_threads_per_atom(parm_system* S, uint32_t tpa) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    // 200: cell-block kernel (shared-memory staging); 1, 2, 4: tiled kernel;
    // 101, 104, 108, 116, 132: gather kernel with 1..32 threads per atom
    if (tpa == 200) {
        if (S->prec != PREC_MIXED) return PARM_OK;
        TRY(S->flush());
        S->want_staged = true;
        return set_staged(S, true);
    }
    const bool tiled = tpa < 100;
    if (tiled && S->prec == PREC_MIXED && !S->c.ntile) return fail(PARM_ERR_ARG, "no tiles in this handle");
    const uint32_t t = tiled ? tpa : tpa - 100;
    if (tiled ? !(t == 1 || t == 2 || t == 4) : !(t == 1 || t == 4 || t == 8 || t == 16 || t == 32))
        return fail(PARM_ERR_ARG, "threads per atom: 200 (cell blocks), 1, 2, 4 (tiled) or 101, 104, 108, 116, "
                                  "132 (gather)");
    if (S->prec != PREC_MIXED) return PARM_OK;
    TRY(S->flush());
    S->want_staged = false;
    S->stg_pending = false;
    TRY(set_staged(S, false));
    if (tiled && !S->c.tiled) {
        launch_tiles(S->c, S->st, 1);   // tiles for the current lists
        TRY(S->sync_status());
    }
    if (S->c.tpa != t || S->c.tiled != (uint32_t)tiled || S->c.unr != 1) {
        S->c.tpa = t;
        S->c.tiled = tiled ? 1u : 0u;
        S->c.unr = 1;
        S->clear_graphs();
    }
    return PARM_OK;
}

int parm_set_active(parm_system* S, const uint8_t* active) {
    if (!S || !active) return fail(PARM_ERR_ARG, "NULL argument");
    TRY(S->flush());
    std::vector<uint32_t> a(S->nsys);
    for (uint32_t s = 0; s < S->nsys; s++) a[s] = active[s] ? 1u : 0u;
    CUDA_TRY(cudaMemcpyAsync(const_cast<uint32_t*>(S->c.active), a.data(), 4 * (size_t)S->nsys,
                             cudaMemcpyHostToDevice, S->st));
    return S->sync_status();
}

int parm_get_threads_per_atom(parm_system* S, uint32_t* tpa) {
    if (!S || !tpa) return fail(PARM_ERR_ARG, "NULL argument");
    if (S->prec != PREC_MIXED) *tpa = 101;
    else if (S->c.staged) *tpa = 200;
    else *tpa = S->c.tiled ? S->c.tpa : 100 + S->c.tpa;
    return PARM_OK;
}

int parm_set_cell_scale(parm_system* S, double scale) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (!(scale >= 1.0 && scale <= 16.0)) return fail(PARM_ERR_ARG, "cell scale must be in [1, 16]");
    TRY(S->flush());
    if (scale == S->cell_scale) return PARM_OK;
    S->cell_scale = scale;
    TRY(S->setup_cells());
    // the next update rebuilds every list on the new grid
    return S->kind >= 0 ? S->request_rebuild_all() : PARM_OK;
}

int parm_debug_stage_cap(parm_system* S, uint32_t cap) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (cap > 4096) return fail(PARM_ERR_ARG, "stage capacity above 4096 atoms");
    TRY(S->flush());
    S->stage_cap_override = cap;
    TRY(S->plan_blocks());
    S->clear_graphs();
    return PARM_OK;
}

int parm_autotune(parm_system* S, uint32_t* tpa_out) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (S->prec != PREC_MIXED || S->kind < 0) {
        if (tpa_out) *tpa_out = S->c.tpa;
        return PARM_OK;
    }
    TRY(S->flush());
    // keep the current forces: the candidates' sums round differently
    CUDA_TRY(cudaMemcpyAsync(S->c.f32b, S->c.f32, sizeof(float4) * (size_t)S->n, cudaMemcpyDeviceToDevice,
                             S->st));
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    // (kind: 2 cell blocks, 1 tiled, 0 gather; threads per atom; neighbours per iteration)
    const uint32_t cands[][3] = {{2, 1, 1}, {1, 1, 1}, {1, 2, 1}, {1, 4, 1}, {0, 1, 1}, {0, 1, 2},
                                 {0, 4, 1}, {0, 8, 1}, {0, 16, 1}};
    const uint32_t keep = S->c.tpa, keep_u = S->c.unr, keep_t = S->c.staged ? 2u : S->c.tiled;
    const bool can_stage = S->stg_ok && !S->stg_pending;
    // both list formats for the comparison
    if (S->c.staged) {
        launch_expand_stg(S->c, S->st);
    } else if (can_stage) {
        launch_compress_stg(S->c, S->st);
    }
    CUDA_TRY(cudaGetLastError());
    float best = 1e30f;
    uint32_t pick = keep, pick_u = keep_u, pick_t = keep_t;
    // the tiled variants rebuild their tiles at every list rebuild: charge
    // that cost, spread over an assumed 10 steps between rebuilds
    float tile_ms = 0.f;
    if (S->c.ntile) {
        launch_tiles(S->c, S->st, 1);
        CUDA_TRY(cudaEventRecord(e0, S->st));
        launch_tiles(S->c, S->st, 1);
        CUDA_TRY(cudaEventRecord(e1, S->st));
        CUDA_TRY(cudaEventSynchronize(e1));
        CUDA_TRY(cudaEventElapsedTime(&tile_ms, e0, e1));
    }
    for (const auto& cu : cands) {
        if (cu[0] == 2 && !can_stage) continue;
        if (cu[0] == 1 && !S->c.ntile) continue;
        S->c.staged = cu[0] == 2 ? 1u : 0u;
        S->c.tiled = cu[0] == 1 ? 1u : 0u;
        S->c.tpa = cu[1];
        S->c.unr = cu[2];
        launch_force32(S->c, S->st, FM_FORCES);   // warm-up
        CUDA_TRY(cudaEventRecord(e0, S->st));
        for (int r = 0; r < 3; r++) launch_force32(S->c, S->st, FM_FORCES);
        CUDA_TRY(cudaEventRecord(e1, S->st));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        ms = ms / 3.f + (cu[0] == 1 ? tile_ms / 10.f : 0.f);
        if (ms < best) {
            best = ms;
            pick_t = cu[0];
            pick = cu[1];
            pick_u = cu[2];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    S->c.staged = pick_t == 2 ? 1u : 0u;
    S->c.tiled = pick_t == 1 ? 1u : 0u;
    S->c.tpa = pick;
    S->c.unr = pick_u;
    S->want_staged = pick_t == 2;
    CUDA_TRY(cudaMemcpyAsync(S->c.f32, S->c.f32b, sizeof(float4) * (size_t)S->n, cudaMemcpyDeviceToDevice,
                             S->st));
    if (pick != keep || pick_u != keep_u || pick_t != keep_t) S->clear_graphs();
    if (tpa_out) *tpa_out = pick_t == 2 ? 2000u : pick_t * 1000 + pick * 10 + pick_u;
    return S->sync_status();
}

int parm_set_graph_steps(parm_system* S, uint32_t k) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (k > 1024) return fail(PARM_ERR_ARG, "steps per graph must be in 0..1024 (0: no graph)");
    S->graph_k = k;
    return PARM_OK;
}

int parm_timing(parm_system* S, int enable) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    S->timing = enable != 0;
    S->t_force = S->t_drift = 0.0;
    S->n_force = 0;
    S->n_rebuild = 0;
    return PARM_OK;
}

int parm_timing_read(parm_system* S, double* force_ms, uint64_t* force_launches, double* drift_ms,
                     uint64_t* rebuilds) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (force_ms) *force_ms = S->t_force;
    if (force_launches) *force_launches = S->n_force;
    if (drift_ms) *drift_ms = S->t_drift;
    if (rebuilds) *rebuilds = S->n_rebuild;
    return PARM_OK;
}

int parm_last_launches(parm_system* S, uint64_t* launches) {
    if (!S || !launches) return fail(PARM_ERR_ARG, "NULL argument");
    *launches = S->last_launches;
    return PARM_OK;
}

int parm_sync(parm_system* S) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    return S->sync_status();
}

void* parm_stream(parm_system* S) { return S ? (void*)S->st : nullptr; }

int parm_host_alloc(void** p, uint64_t bytes) {
    if (!p) return fail(PARM_ERR_ARG, "NULL argument");
    CUDA_TRY(cudaMallocHost(p, bytes));
    return PARM_OK;
}

int parm_host_free(void* p) {
    CUDA_TRY(cudaFreeHost(p));
    return PARM_OK;
}

int parm_debug_remainder(const double* d, const double* L, double* out, uint32_t n) {
    if (!d || !L || !out) return fail(PARM_ERR_ARG, "NULL argument");
    if (n == 0) return PARM_OK;
    double* buf = nullptr;
    CUDA_TRY(cudaMalloc(&buf, 24 * (size_t)n));
    cudaMemcpy(buf, d, 8 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(buf + n, L, 8 * (size_t)n, cudaMemcpyHostToDevice);
    launch_remainder_test(buf, buf + n, buf + 2 * (size_t)n, n, 0);
    cudaError_t e = cudaMemcpy(out, buf + 2 * (size_t)n, 8 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(PARM_ERR_CUDA, cudaGetErrorString(e));
    return PARM_OK;
}

// ---- conjugate-gradient minimisers ----
static constexpr int kNlcgWords = (int)(sizeof(NlcgSys) / 8);

static int nlcg_read(parm_system* S, std::vector<double>& hp) {
    hp.assign((size_t)S->nsys * kNlcgWords, 0.0);
    CUDA_TRY(cudaStreamSynchronize(S->st));
    CUDA_TRY(cudaMemcpy(hp.data(), S->c.nlcg, sizeof(NlcgSys) * S->nsys, cudaMemcpyDeviceToHost));
    return PARM_OK;
}

static int nlcg_write(parm_system* S, const std::vector<double>& hp) {
    CUDA_TRY(cudaStreamSynchronize(S->st));
    CUDA_TRY(cudaMemcpy(S->c.nlcg, hp.data(), sizeof(NlcgSys) * S->nsys, cudaMemcpyHostToDevice));
    return PARM_OK;
}

static int nlcg_check_params(const double* p, bool boxed) {
    if (!(p[0] == p[0]) || !(p[3] == p[3]) || !(p[4] >= 0.0 && p[4] <= 1e6) || p[4] != std::floor(p[4]))
        return fail(PARM_ERR_ARG, "minimiser parameters: dt and kmax must be numbers, secmax an integer "
                                  "in [0, 1e6]");
    if (boxed && !(p[2] > 0.0)) return fail(PARM_ERR_ARG, "CollectionNLCG: kappa must be > 0");
    return PARM_OK;
}

int parm_nlcg_init(parm_system* S, int boxed, const double* params) {
    if (!S || !params) return fail(PARM_ERR_ARG, "NULL argument");
    for (uint32_t s = 0; s < S->nsys; s++) TRY(nlcg_check_params(params + (size_t)s * PARM_NLCG_NPARAM, boxed != 0));
    if (S->prec == PREC_MIXED && (S->c.staged || S->c.tiled || S->want_staged))
        TRY(parm_set_threads_per_atom(S, 101));   // the minimiser uses the per-atom lists
    TRY(S->flush());
    CUDA_TRY(cudaStreamSynchronize(S->st));
    if (!S->nlcg_mem) {
        const size_t bytes = sizeof(NlcgSys) * (size_t)S->nsys + 8 * (size_t)S->nsys + 16;
        CUDA_TRY(cudaMalloc(&S->nlcg_mem, bytes));
        CUDA_TRY(cudaMemset(S->nlcg_mem, 0, bytes));
        char* b = static_cast<char*>(S->nlcg_mem);
        S->c.nlcg = reinterpret_cast<NlcgSys*>(b);
        S->c.nlcg_step = reinterpret_cast<uint32_t*>(b + sizeof(NlcgSys) * (size_t)S->nsys);
        S->c.nlcg_loop = S->c.nlcg_step + S->nsys;
        S->c.nlcg_any = S->c.nlcg_loop + S->nsys;
    }
    // a fresh minimiser: the parameters given, every state variable 0
    // (the reference constructors' initialiser lists)
    std::vector<double> hp((size_t)S->nsys * kNlcgWords, 0.0);
    for (uint32_t s = 0; s < S->nsys; s++)
        for (int q = 0; q < PARM_NLCG_NPARAM; q++)
            hp[(size_t)s * kNlcgWords + q] = params[(size_t)s * PARM_NLCG_NPARAM + q];
    TRY(nlcg_write(S, hp));
    S->nlcg_boxed = boxed != 0;
    S->c.nlcg_boxed = boxed ? 1u : 0u;
    S->clear_graphs();
    return PARM_OK;
}

int parm_nlcg_set_params(parm_system* S, const double* params) {
    if (!S || !params) return fail(PARM_ERR_ARG, "NULL argument");
    if (!S->c.nlcg) return fail(PARM_ERR_RUNTIME, "parm_nlcg_init has not been called on this handle");
    for (uint32_t s = 0; s < S->nsys; s++)
        TRY(nlcg_check_params(params + (size_t)s * PARM_NLCG_NPARAM, S->nlcg_boxed));
    std::vector<double> hp;
    TRY(nlcg_read(S, hp));
    for (uint32_t s = 0; s < S->nsys; s++)
        for (int q = 0; q < PARM_NLCG_NPARAM; q++)
            hp[(size_t)s * kNlcgWords + q] = params[(size_t)s * PARM_NLCG_NPARAM + q];
    return nlcg_write(S, hp);
}

int parm_nlcg_get_state(parm_system* S, double* state) {
    if (!S || !state) return fail(PARM_ERR_ARG, "NULL argument");
    if (!S->c.nlcg) return fail(PARM_ERR_RUNTIME, "parm_nlcg_init has not been called on this handle");
    std::vector<double> hp;
    TRY(nlcg_read(S, hp));
    for (uint32_t s = 0; s < S->nsys; s++)
        for (int q = 0; q < PARM_NLCG_NSTATE; q++)
            state[(size_t)s * PARM_NLCG_NSTATE + q] = hp[(size_t)s * kNlcgWords + PARM_NLCG_NPARAM + q];
    return PARM_OK;
}

int parm_nlcg_set_state(parm_system* S, const double* state) {
    if (!S || !state) return fail(PARM_ERR_ARG, "NULL argument");
    if (!S->c.nlcg) return fail(PARM_ERR_RUNTIME, "parm_nlcg_init has not been called on this handle");
    std::vector<double> hp;
    TRY(nlcg_read(S, hp));
    for (uint32_t s = 0; s < S->nsys; s++)
        for (int q = 0; q < PARM_NLCG_NSTATE; q++)
            hp[(size_t)s * kNlcgWords + PARM_NLCG_NPARAM + q] = state[(size_t)s * PARM_NLCG_NSTATE + q];
    return nlcg_write(S, hp);
}

// CollectionNLCG::set_forces(constraints_and_a, true) (src/collection.cpp:534-566);
// CollectionNLCGV: Collection::set_forces (src/collection.cpp:159-179)
static int nlcg_set_forces_impl(parm_system* S, bool c_and_a) {
    DevCtx cb, cs;
    S->nlcg_ctx(cb, cs);
    if (!S->nlcg_boxed) {
        const int mode = c_and_a ? FM_FORCES_A : FM_FORCES;
        if (S->prec == PREC_FP64) launch_force64(cb, S->st, mode);
        else launch_force32(cb, S->st, mode);
        CUDA_TRY(cudaGetLastError());
        return PARM_OK;
    }
    CUDA_TRY(cudaMemcpyAsync(S->c.nlcg_step, S->c.active, 4 * (size_t)S->nsys, cudaMemcpyDeviceToDevice, S->st));
    S->nlcg_forces(cb, cs, S->st);
    launch_nlcg_atoms(cb, S->st, NA_IMMOBILE_A);
    if (c_and_a) {
        launch_nlcg_atoms(cb, S->st, NA_SETF);
        launch_nlcg_terms(cb, S->st, NT_FA_FF, S->c.active);
        launch_sys_reduce(cb, S->st, 2);
        launch_nlcg_ctl(cb, S->st, NP_SETF, 0, 0);
    }
    CUDA_TRY(cudaGetLastError());
    return PARM_OK;
}

int parm_nlcg_set_forces(parm_system* S, int constraints_and_a) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    TRY(S->nlcg_prepare());
    TRY(nlcg_set_forces_impl(S, constraints_and_a != 0));
    return S->sync_status();
}

int parm_nlcg_reset(parm_system* S) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    TRY(S->nlcg_prepare());
    DevCtx cb, cs;
    S->nlcg_ctx(cb, cs);
    if (S->nlcg_boxed) {
        // CollectionNLCG::reset (collection.cpp:525-532)
        TRY(nlcg_set_forces_impl(S, true));
        launch_nlcg_atoms(cb, S->st, NA_RESET);
        launch_nlcg_ctl(cb, S->st, NP_RESET, 0, 0);
    } else {
        // CollectionNLCGV::reset (collection.cpp:977-988)
        launch_nlcg_ctl(cb, S->st, NP_RESET, 0, 0);
        TRY(nlcg_set_forces_impl(S, false));
        launch_nlcg_atoms(cb, S->st, NA_DESCEND);
    }
    CUDA_TRY(cudaGetLastError());
    return S->sync_status();
}

int parm_nlcg_descend(parm_system* S) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    TRY(S->nlcg_prepare());
    DevCtx cb, cs;
    S->nlcg_ctx(cb, cs);
    // descend (collection.cpp:811-829, 990-1005): forces, v = a = f, stepx(dt), trackers
    TRY(nlcg_set_forces_impl(S, false));
    launch_nlcg_atoms(cb, S->st, NA_DESCEND);
    launch_nlcg_ctl(cb, S->st, NP_DESCEND, 0, 0);
    launch_nlcg_stepx(cb, S->st);
    launch_nlcg_box(cb, S->st);
    TRY(S->nlcg_update_trackers(cb, false));
    TRY(S->sync_status());
    return S->nlcg_sync_boxes();
}

int parm_nlcg_timestep(parm_system* S, uint32_t nsteps) {
    if (!S) return fail(PARM_ERR_ARG, "NULL handle");
    if (nsteps == 0) return PARM_OK;
    return S->nlcg_run(nsteps);
}

int parm_get_boxes(parm_system* S, double* L) {
    if (!S || !L) return fail(PARM_ERR_ARG, "NULL argument");
    std::copy(S->L.begin(), S->L.end(), L);
    return PARM_OK;
}

int parm_debug_philox(const uint32_t* in, uint32_t* out, uint32_t n) {
    if (!in || !out) return fail(PARM_ERR_ARG, "NULL argument");
    if (n == 0) return PARM_OK;
    uint32_t* buf = nullptr;
    CUDA_TRY(cudaMalloc(&buf, 40 * (size_t)n));
    cudaError_t e = cudaMemcpy(buf, in, 24 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_philox_test(buf, buf + 6 * (size_t)n, n, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, buf + 6 * (size_t)n, 16 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(PARM_ERR_CUDA, cudaGetErrorString(e));
    return PARM_OK;
}

int parm_debug_fpbits(const double* d, const float* f, uint32_t n, float* d2f, double* f2d) {
    if (!d || !f || !d2f || !f2d) return fail(PARM_ERR_ARG, "NULL argument");
    if (n == 0) return PARM_OK;
    char* buf = nullptr;
    CUDA_TRY(cudaMalloc(&buf, 24 * (size_t)n));
    double* dd = reinterpret_cast<double*>(buf);
    double* df2d = dd + n;
    float* df = reinterpret_cast<float*>(df2d + n);
    float* dd2f = df + n;
    cudaError_t e = cudaMemcpy(dd, d, 8 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(df, f, 4 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_fpbits_test(dd, df, n, dd2f, df2d, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(d2f, dd2f, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f2d, df2d, 8 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(PARM_ERR_CUDA, cudaGetErrorString(e));
    return PARM_OK;
}

int parm_debug_normals(uint64_t seed, uint32_t sys, uint64_t step, uint32_t natoms, double* out) {
    if (!out) return fail(PARM_ERR_ARG, "NULL argument");
    if (natoms == 0) return PARM_OK;
    double* buf = nullptr;
    CUDA_TRY(cudaMalloc(&buf, 48 * (size_t)natoms));
    launch_normals_test(splitmix64(seed + sys), step, natoms, buf, 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, buf, 48 * (size_t)natoms, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return fail(PARM_ERR_CUDA, cudaGetErrorString(e));
    return PARM_OK;
}

}  // extern "C"
