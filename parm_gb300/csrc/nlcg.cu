// Conjugate-gradient minimisers on the GPU, batched over systems:
//   CollectionNLCG  (src/collection.hpp:400-475, src/collection.cpp:494-829):
//     positions s_i and kappa ln V, energy U + P0 V; stepx scales positions
//     and box by exp(dx vl / (kappa d)) and moves them by v dx;
//   CollectionNLCGV (src/collection.hpp:490-566, src/collection.cpp:877-1168):
//     positions only, fixed box.
// Every system keeps its own minimiser state (NlcgSys) in device memory and
// runs its own secant line search; one launch of each kernel serves all
// systems.  Per-system scalar decisions are taken by k_nlcg_ctl (one thread
// per system); per-atom work by k_nlcg_stepx / k_nlcg_atoms / k_nlcg_terms;
// the sums (fdotv, vdotv, fdota, the virial) by the deterministic two-pass
// per-system reductions of integrate.cu.  The secant loop runs inside a CUDA
// graph as a conditional WHILE node whose condition k_nlcg_ctl sets while any
// system is still searching, so a time step needs no host round trip.
//
// Compiled with -fmad=false: the update formulas round like the reference's
// unfused FP64 code.  The sums are parallel, so the scalars (and the
// trajectories through them) agree with the reference to rounding, not bit
// for bit.
#include "parm_ctx.cuh"

namespace parm {

__device__ __forceinline__ bool mobile_cg(double m) { return !(m <= 0.0 || isinf(m)); }

template <int ND>
__device__ __forceinline__ void ld3(const void* p, uint32_t i, double* o) {
    using V = typename DVec<ND>::T;
    const V t = static_cast<const V*>(p)[i];
    const double* q = reinterpret_cast<const double*>(&t);
#pragma unroll
    for (int d = 0; d < ND; d++) o[d] = q[d];
}

template <int ND>
__device__ __forceinline__ void st3(void* p, uint32_t i, const double* o) {
    using V = typename DVec<ND>::T;
    V t;
    double* q = reinterpret_cast<double*>(&t);
#pragma unroll
    for (int d = 0; d < (int)(sizeof(V) / 8); d++) q[d] = d < ND ? o[d] : 0.0;
    static_cast<V*>(p)[i] = t;
}

// the force of atom i in FP64 (the mixed path keeps forces in FP32)
template <int ND>
__device__ __forceinline__ void ldf(const DevCtx& c, uint32_t i, double* f) {
    if (c.prec == PREC_MIXED) {
        const float4 q = c.f32[i];
        f[0] = q.x;
        f[1] = q.y;
        if (ND == 3) f[2] = q.z;
    } else {
        ld3<ND>(c.f, i, f);
    }
}

// Eigen's fixed-size dot: ((a0 b0 + a1 b1) + a2 b2)
template <int ND>
__device__ __forceinline__ double dot(const double* a, const double* b) {
    double s = a[0] * b[0] + a[1] * b[1];
    if constexpr (ND == 3) s = s + a[2] * b[2];
    return s;
}

// FP32 position view (coarse X = trunc(8 x) / 8 and fine x - X), as written
// by every kernel that moves atoms; the list diameter in A.w is kept
template <int ND>
__device__ __forceinline__ void posq_store(const DevCtx& c, uint32_t i, const double* xs) {
    float4 A = c.pos[2 * (size_t)i], B;
    float* Ap = &A.x;
    float* Bp = &B.x;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (d < ND) {
            const double t = trunc(xs[d] * 8.0) * 0.125;
            Ap[d] = (float)t;
            Bp[d] = (float)(xs[d] - t);
        } else {
            Ap[d] = 0.f;
            Bp[d] = 0.f;
        }
    }
    B.w = 0.f;
    c.pos[2 * (size_t)i] = A;
    c.pos[2 * (size_t)i + 1] = B;
}

// OriginBox::V (src/box.hpp:112) and CollectionNLCG::get_length_squared
// (src/collection.cpp:641-649)
template <int ND>
__device__ __forceinline__ double box_volume(const SysConst& S) {
    double V = S.L[0] * S.L[1];
    if constexpr (ND == 3) V = V * S.L[2];
    return V;
}
template <int ND>
__device__ __forceinline__ double length_sq(const SysConst& S) {
    return ND == 3 ? pow(box_volume<ND>(S), 2.0 / 3.0) : box_volume<ND>(S);
}

// ---------------------------------------------------------------------------
// stepx: CollectionNLCG::stepx (collection.cpp:621-639): every atom x *= Lfac,
// x += v dx; CollectionNLCGV::stepx (900-908): mobile atoms x += v dx.  The
// set_forces that follows in CollectionNLCG (Collection::
// set_forces_get_pressure, collection.cpp:181-208) zeroes the acceleration of
// immobile atoms; that is done here as well.
// ---------------------------------------------------------------------------
template <int ND, bool BOXED>
__global__ void __launch_bounds__(BLOCK) k_nlcg_stepx(DevCtx c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const uint32_t s = c.atom_sys[i];
    if (!c.nlcg_step[s]) return;
    const NlcgSys& G = c.nlcg[s];
    const double m = c.m[i];
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0};
    ld3<ND>(c.x, i, x);
    ld3<ND>(c.v, i, v);
    if (BOXED) {
        const double lf = G.lfac, dx = G.dx;
#pragma unroll
        for (int d = 0; d < ND; d++) {
            x[d] = x[d] * lf;
            x[d] = x[d] + v[d] * dx;
        }
        if (!mobile_cg(m)) {
            const double z[3] = {0, 0, 0};
            st3<ND>(c.a, i, z);
        }
    } else {
        if (!mobile_cg(m)) return;
        const double dx = G.dx;
#pragma unroll
        for (int d = 0; d < ND; d++) x[d] = x[d] + v[d] * dx;
    }
    st3<ND>(c.x, i, x);
    posq_store<ND>(c, i, x);
}

// ---------------------------------------------------------------------------
// OriginBox::resize(Lfac) (src/box.hpp:125-128) of the systems that stepped,
// with every quantity derived from the box; when a cell becomes narrower than
// the list radius the system's grid shrinks in place (fewer cells along that
// axis; its bucket range keeps its size, the unused tail is zeroed).  A grid
// only shrinks here; the host regrids wider boxes between calls.
// ---------------------------------------------------------------------------
template <int ND>
__global__ void k_nlcg_box(DevCtx c) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= c.nsys || !c.nlcg_step[s]) return;
    SysConst& S = const_cast<SysConst&>(c.sys[s]);
    const double f = c.nlcg[s].lfac;
    const double w = S.cellmin;
    const uint32_t ncell_old = S.ncell;
    bool regrid = false;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        const double l = S.L[d] * f;
        S.L[d] = l;
        S.invL[d] = 1.0 / l;
        S.halfL[d] = 0.5 * l;
        S.Lhi[d] = (float)l;
        S.Llo[d] = (float)(l - (double)S.Lhi[d]);
        S.invLf[d] = (float)(1.0 / l);
        const double l8 = rint(l * 8.0) * 0.125;
        S.L8[d] = (float)l8;
        S.Lr8[d] = (float)(l - l8);
        if (S.nc[d] > 1 && w > 0.0 && l / S.nc[d] < w) {
            const double q = floor(l / w);
            S.nc[d] = q >= 3.0 ? (int)q : 1;
            regrid = true;
        }
        S.cellw_inv[d] = (float)(S.nc[d] / l);
        S.cellw[d] = l / S.nc[d];
        S.cellw32[d] = (float)S.cellw[d];
    }
    if (regrid) {
        S.ncell = (uint32_t)(S.nc[0] * S.nc[1] * S.nc[2]);
        // counts left in buckets past the new non-member bucket would be
        // scanned into nothing but must not carry stale sums
        const uint32_t b0 = c.bucket_off[s];
        for (uint32_t b = S.ncell + 1; b <= ncell_old; b++) c.cell_count[b0 + b] = 0u;
        // the current lists index atoms, not cells: they stay valid, and the
        // next rebuild (when the displacement test asks for one) bins on this grid
    }
}

// ---------------------------------------------------------------------------
// per-atom inputs of the per-system sums (component-major in red), mobile
// atoms of systems flagged in `mask` only:
//   NT_FV    f . v       (fdotv)
//   NT_VV    v . v       (vdotv)
//   NT_FA_FF f . a, f . f (fdota before and after a = f)
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(BLOCK) k_nlcg_terms(DevCtx c, int what, const uint32_t* mask) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const uint32_t s = c.atom_sys[i];
    double t0 = 0.0, t1 = 0.0;
    if (mask[s] && mobile_cg(c.m[i])) {
        double f[3] = {0, 0, 0}, q[3] = {0, 0, 0};
        if (what == NT_VV) {
            ld3<ND>(c.v, i, q);
            t0 = dot<ND>(q, q);
        } else {
            ldf<ND>(c, i, f);
            if (what == NT_FV) {
                ld3<ND>(c.v, i, q);
                t0 = dot<ND>(f, q);
            } else {
                ld3<ND>(c.a, i, q);
                t0 = dot<ND>(f, q);
                t1 = dot<ND>(f, f);
            }
        }
    }
    c.red[i] = t0;
    if (what == NT_FA_FF) c.red[(size_t)c.n + i] = t1;
}

// ---------------------------------------------------------------------------
// per-atom updates of the direction (active systems)
// ---------------------------------------------------------------------------
template <int ND, bool BOXED>
__global__ void __launch_bounds__(BLOCK) k_nlcg_atoms(DevCtx c, int what) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const uint32_t s = c.atom_sys[i];
    if (!c.active[s]) return;
    const bool mob = mobile_cg(c.m[i]);
    const double z[3] = {0, 0, 0};
    double f[3] = {0, 0, 0};
    if (what == NA_FINISH) {
        // CollectionNLCG::timestep, collection.cpp:784-808: a = f, v = a + v betaused
        // (immobile atoms: a = v = 0); CollectionNLCGV, 1142-1161: every atom
        if (BOXED && !mob) {
            st3<ND>(c.a, i, z);
            st3<ND>(c.v, i, z);
            return;
        }
        const double bu = c.nlcg[s].betaused;
        double v[3] = {0, 0, 0};
        ldf<ND>(c, i, f);
        ld3<ND>(c.v, i, v);
#pragma unroll
        for (int d = 0; d < ND; d++) v[d] = f[d] + v[d] * bu;
        st3<ND>(c.a, i, f);
        st3<ND>(c.v, i, v);
    } else if (what == NA_SETF) {
        // CollectionNLCG::set_forces(true, ...), collection.cpp:553-563
        if (!mob) {
            st3<ND>(c.a, i, z);
            st3<ND>(c.v, i, z);
            return;
        }
        ldf<ND>(c, i, f);
        st3<ND>(c.a, i, f);
        st3<ND>(c.v, i, f);
    } else if (what == NA_RESET) {
        // CollectionNLCG::reset, collection.cpp:528-530: v = a for every atom
        double a[3] = {0, 0, 0};
        ld3<ND>(c.a, i, a);
        st3<ND>(c.v, i, a);
    } else if (what == NA_DESCEND) {
        // descend (collection.cpp:814-822, 993-1000) and CollectionNLCGV::reset
        // (980-987): v = a = f for mobile atoms
        if (!mob) return;
        ldf<ND>(c, i, f);
        st3<ND>(c.a, i, f);
        st3<ND>(c.v, i, f);
    } else if (what == NA_IMMOBILE_A) {
        if (!mob) st3<ND>(c.a, i, z);
    }
}

// ---------------------------------------------------------------------------
// per-system decisions (one thread per system); sysout holds the sums of the
// preceding reduction
// ---------------------------------------------------------------------------
template <int ND, bool BOXED>
__global__ void k_nlcg_ctl(DevCtx c, int phase, int use_cond, cudaGraphConditionalHandle handle) {
    __shared__ int sany;
    if (threadIdx.x == 0) sany = 0;
    __syncthreads();
    int any = 0;
    const double kd = (double)ND;
    for (uint32_t s = threadIdx.x; s < c.nsys; s += blockDim.x) {
        NlcgSys& G = c.nlcg[s];
        const SysConst& S = c.sys[s];
        const bool act = c.active[s] != 0;
        const double lsq = BOXED ? length_sq<ND>(S) : 1.0;
        switch (phase) {
            case NP_BEGIN:   // stepx(dt)
                if (act) {
                    G.dx = G.dt;
                    G.lfac = BOXED ? exp(G.dx * G.vl / (G.kappa * kd)) : 1.0;
                }
                c.nlcg_step[s] = act ? 1u : 0u;
                break;
            case NP_FL:      // CollectionNLCG::set_forces(.., true), collection.cpp:536-541
                if (BOXED && c.nlcg_step[s]) {
                    const double interacP = c.sysout[s];
                    G.fl = ((interacP / kd) - (G.P0 * box_volume<ND>(S))) / G.kappa;
                }
                break;
            case NP_ETA0:    // eta0 = -fdotv() (collection.cpp:701); stepx(-dt) next
                if (act) {
                    const double fv = BOXED ? c.sysout[s] / lsq + G.fl * G.vl : c.sysout[s];
                    G.eta0 = -fv;
                    G.dx = -G.dt;
                    G.lfac = BOXED ? exp(G.dx * G.vl / (G.kappa * kd)) : 1.0;
                }
                c.nlcg_step[s] = act ? 1u : 0u;
                break;
            case NP_LOOPINIT:   // collection.cpp:703-711
                if (act) {
                    G.vdv = BOXED ? c.sysout[s] / lsq + G.vl * G.vl : c.sysout[s];
                    G.alpha = -G.dt;
                    G.dxsum = 0.0;
                    G.sec = 0.0;
                    G.iters = 0.0;
                }
                c.nlcg_loop[s] = (act && G.secmax > 0.0) ? 1u : 0u;
                c.nlcg_step[s] = 0u;
                any |= c.nlcg_loop[s] ? 1 : 0;
                break;
            case NP_PRE: {   // collection.cpp:716-773 up to stepx(alpha)
                c.nlcg_step[s] = 0u;
                if (!c.nlcg_loop[s]) break;
                const double fv = BOXED ? c.sysout[s] / lsq + G.fl * G.vl : c.sysout[s];
                const double eta = -fv;
                G.eta = eta;
                double alphafac = -eta / fabs(G.eta0 - eta);
                if (fabs(G.eta0 - eta) <= 1e-12 * fabs(eta)) {
                    alphafac = G.alphamax > 0 ? G.alphamax : 1.1;
                    G.sec = G.sec > 0 ? G.sec * 2 - 1 : 1;
                }
                if (G.alphamax > 0 && alphafac > G.alphamax) alphafac = G.alphamax;
                if (G.alphamax > 0 && alphafac < -G.alphamax) alphafac = -G.alphamax;
                G.alpha = fabs(G.alpha) * alphafac;
                const double newdxsum = fabs(G.dxsum + G.alpha);
                if (G.dxmax > 0 && newdxsum > G.dxmax) {
                    G.k = 0;
                    c.nlcg_loop[s] = 0u;
                    break;
                }
                if (BOXED) {
                    const double dVoverV = expm1(fabs(G.dxsum + G.alpha) * G.vl / (G.kappa * kd));
                    if (G.maxdV > 0 && dVoverV > G.maxdV) {
                        G.k = 0;
                        c.nlcg_loop[s] = 0u;
                        break;
                    }
                }
                G.dxsum += G.alpha;
                G.dx = G.alpha;
                G.lfac = BOXED ? exp(G.dx * G.vl / (G.kappa * kd)) : 1.0;
                c.nlcg_step[s] = 1u;
                break;
            }
            case NP_POST:    // collection.cpp:774-790 and the loop increment
                if (c.nlcg_step[s]) {
                    G.eta0 = G.eta;
                    bool brk = false;
                    if (G.alpha * G.alpha * G.vdv < G.seceps * G.seceps) brk = true;
                    else if ((G.sec > 1) && (G.afrac > 0) && (fabs(G.alpha) < fabs(G.dxsum)) &&
                             (fabs(G.alpha) / fabs(G.dxsum) < G.afrac))
                        brk = true;
                    else if (G.stepmax > 0 && G.dxsum * G.dxsum * G.vdv > G.stepmax * G.stepmax) {
                        G.k = 0;
                        brk = true;
                    }
                    if (brk) {
                        c.nlcg_loop[s] = 0u;
                    } else {
                        G.sec += 1;
                        if (!(G.sec < G.secmax)) c.nlcg_loop[s] = 0u;
                    }
                    // sec grows by at least one per iteration, so the loop ends
                    // within secmax iterations; the count bounds it regardless
                    G.iters += 1;
                    if (!(G.iters < G.secmax)) c.nlcg_loop[s] = 0u;
                }
                c.nlcg_step[s] = 0u;
                any |= c.nlcg_loop[s] ? 1 : 0;
                break;
            case NP_FINISH:  // collection.cpp:792-809 (sysout: fdota before, after a = f)
                if (act) {
                    G.alphavmax = sqrt(G.alpha * G.alpha * G.vdv);
                    const double Kold = G.Knew;
                    const double Kmid = BOXED ? c.sysout[2 * s] / lsq + G.fl * G.al : c.sysout[2 * s];
                    G.al = G.fl;
                    G.Knew = BOXED ? c.sysout[2 * s + 1] / lsq + G.fl * G.al : c.sysout[2 * s + 1];
                    G.beta = (G.Knew - Kmid) / Kold;
                    G.betaused = G.beta;
                    G.k += 1;
                    if (G.k >= G.kmax || isinf(G.betaused) || isnan(G.betaused) || G.betaused <= 0) {
                        G.k = 0;
                        G.betaused = 0;
                    } else if (G.betaused > 1) {
                        G.betaused = 1;
                    }
                    if (BOXED) G.vl = G.al + G.betaused * G.vl;
                }
                break;
            case NP_SETF:    // set_forces(true, true): al = vl = fl; Knew = fdota() with a = f
                if (act) {
                    if (BOXED) {
                        G.al = G.fl;
                        G.vl = G.fl;
                    }
                    G.Knew = BOXED ? c.sysout[2 * s + 1] / lsq + G.fl * G.al : c.sysout[2 * s + 1];
                }
                break;
            case NP_RESET:   // reset(): k = 0 (and vl = al)
                if (act) {
                    G.k = 0;
                    if (BOXED) G.vl = G.al;
                }
                break;
            case NP_DESCEND:  // descend(): al = vl = fl, then stepx(dt)
                if (act) {
                    if (BOXED) {
                        G.al = G.fl;
                        G.vl = G.fl;
                    }
                    G.dx = G.dt;
                    G.lfac = BOXED ? exp(G.dx * G.vl / (G.kappa * kd)) : 1.0;
                }
                c.nlcg_step[s] = act ? 1u : 0u;
                break;
            default:
                break;
        }
    }
    if (any) atomicOr(&sany, 1);
    __syncthreads();
    if (threadIdx.x == 0 && (phase == NP_LOOPINIT || phase == NP_POST)) {
        *c.nlcg_any = (uint32_t)sany;
        if (use_cond) cudaGraphSetConditional(handle, sany ? 1u : 0u);
    }
}

// ---------------------------------------------------------------------------
void launch_nlcg_stepx(const DevCtx& c, cudaStream_t s) {
    const unsigned g = grid_for(c.n);
    if (c.nd == 3) {
        if (c.nlcg_boxed) k_nlcg_stepx<3, true><<<g, BLOCK, 0, s>>>(c);
        else k_nlcg_stepx<3, false><<<g, BLOCK, 0, s>>>(c);
    } else {
        if (c.nlcg_boxed) k_nlcg_stepx<2, true><<<g, BLOCK, 0, s>>>(c);
        else k_nlcg_stepx<2, false><<<g, BLOCK, 0, s>>>(c);
    }
}

void launch_nlcg_box(const DevCtx& c, cudaStream_t s) {
    if (!c.nlcg_boxed) return;
    const unsigned g = (c.nsys + 127) / 128;
    if (c.nd == 3) k_nlcg_box<3><<<g, 128, 0, s>>>(c);
    else k_nlcg_box<2><<<g, 128, 0, s>>>(c);
}

void launch_nlcg_ctl(const DevCtx& c, cudaStream_t s, int phase, int use_cond, unsigned long long handle) {
    const unsigned t = c.nsys >= 1024 ? 1024u : ((c.nsys + 31) / 32) * 32;
    const auto h = (cudaGraphConditionalHandle)handle;
    if (c.nd == 3) {
        if (c.nlcg_boxed) k_nlcg_ctl<3, true><<<1, t, 0, s>>>(c, phase, use_cond, h);
        else k_nlcg_ctl<3, false><<<1, t, 0, s>>>(c, phase, use_cond, h);
    } else {
        if (c.nlcg_boxed) k_nlcg_ctl<2, true><<<1, t, 0, s>>>(c, phase, use_cond, h);
        else k_nlcg_ctl<2, false><<<1, t, 0, s>>>(c, phase, use_cond, h);
    }
}

void launch_nlcg_terms(const DevCtx& c, cudaStream_t s, int what, const uint32_t* mask) {
    const unsigned g = grid_for(c.n);
    if (c.nd == 3) k_nlcg_terms<3><<<g, BLOCK, 0, s>>>(c, what, mask);
    else k_nlcg_terms<2><<<g, BLOCK, 0, s>>>(c, what, mask);
}

void launch_nlcg_atoms(const DevCtx& c, cudaStream_t s, int what) {
    const unsigned g = grid_for(c.n);
    if (c.nd == 3) {
        if (c.nlcg_boxed) k_nlcg_atoms<3, true><<<g, BLOCK, 0, s>>>(c, what);
        else k_nlcg_atoms<3, false><<<g, BLOCK, 0, s>>>(c, what);
    } else {
        if (c.nlcg_boxed) k_nlcg_atoms<2, true><<<g, BLOCK, 0, s>>>(c, what);
        else k_nlcg_atoms<2, false><<<g, BLOCK, 0, s>>>(c, what);
    }
}

}  // namespace parm
