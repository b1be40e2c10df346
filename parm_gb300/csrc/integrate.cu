// Position/velocity integration, host-layout transfers and per-system
// reductions.  All FP64 arithmetic here follows the reference's expression
// order and is compiled with -fmad=false so that it rounds exactly like the
// reference's unfused CPU code.
//
// Reference time-step loops (wackywendell/parm src/collection.cpp):
//   CollectionVerlet::timestep  442-469  (first loop: drift + half kick)
//   CollectionDamped::timestep  356-381  (first loop)
//   CollectionSol::timestep     265-322  (first loop, BivariateGauss noise)
// The second half of step k (a = f/m and the final velocity update) is fused
// with the first half of step k+1 in k_kickdrift; a call ends with k_kick.
#include "fpbits.cuh"
#include "parm_check.cuh"

namespace parm {

__device__ __forceinline__ bool mobile(double m) { return !(m <= 0.0 || isinf(m)); }

// the same test on the bit pattern (integer instructions, not the FP64 pipe):
// NaN -> mobile; +-0, negative, +-inf -> not
__device__ __forceinline__ bool mobile_bits(double m) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(m);
    const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
    return mag > 0x7FF0000000000000ull || ((b >> 63) == 0ull && mag != 0ull && mag != 0x7FF0000000000000ull);
}

__device__ __forceinline__ void posq_split2(double x, float& X, float& xf) {
    double t = trunc(x * 8.0) * 0.125;
    X = (float)t;
    xf = (float)(x - t);
}

// ---- counter-based Gaussian noise (Philox4x32-10 + Box-Muller) ----
__device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    unsigned long long v = ((unsigned long long)(a >> 5) << 26) | (unsigned long long)(b >> 6);
    return ((double)v + 0.5) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ void normals6(unsigned long long seed, unsigned long long step,
                                         uint32_t atom, double out[6]) {
#pragma unroll
    for (uint32_t blk = 0; blk < 3; blk++) {
        uint32_t c[4] = {atom, (uint32_t)step, (uint32_t)(step >> 32), blk};
        philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        double u1 = u53(c[0], c[1]);
        double u2 = u53(c[2], c[3]);
        double r = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincos(6.283185307179586 * u2, &sn, &cs);
        out[2 * blk] = r * cs;
        out[2 * blk + 1] = r * sn;
    }
}

template <int ND>
__device__ __forceinline__ void store_posq(const DevCtx& c, uint32_t i, const double* xs) {
    float4 A = c.pos[2 * (size_t)(i)], B;
    posq_split2(xs[0], A.x, B.x);
    posq_split2(xs[1], A.y, B.y);
    if constexpr (ND == 3) posq_split2(xs[2], A.z, B.z); else { A.z = 0.f; B.z = 0.f; }
    B.w = 0.f;
    c.pos[2 * (size_t)(i)] = A;
    c.pos[2 * (size_t)(i) + 1] = B;
    if (c.staged) c.rec[i] = make_record(A, B, c.rframe[i]);
}

// Second half of the previous step (the reference's loop after set_forces):
// a = f/m and the final velocity update.  Mobility tests as in the reference:
// Verlet and Damped skip m <= 0 or inf; Sol tests m == 0 or inf.
template <int ND, int MODE, bool MIXED>
__device__ __forceinline__ void kick(const DevCtx& c, uint32_t i, double m, double* a, double* v) {
    const StepParams& P = *c.params;
    double f[3] = {0.0, 0.0, 0.0};
    float fm[3] = {0.f, 0.f, 0.f};
    if constexpr (MIXED) {
        const float4 q = c.f32[i];
        fm[0] = q.x;
        fm[1] = q.y;
        fm[2] = q.z;
    } else {
        using V = typename DVec<ND>::T;
        V fv = static_cast<const V*>(c.f)[i];
        const double* fp = reinterpret_cast<const double*>(&fv);
#pragma unroll
        for (int d = 0; d < ND; d++) f[d] = fp[d];
    }
    const bool sol = (MODE == DM_SOL);
    const bool has_a = sol ? !(m == 0.0 || isinf(m)) : mobile(m);
    if (!has_a) {
#pragma unroll
        for (int d = 0; d < ND; d++) {
            a[d] = 0.0;
            if (sol) v[d] = 0.0;
        }
        return;
    }
    if constexpr (MIXED) {
        const float im = mobile(m) ? c.invm32[i] : (float)(1.0 / m);
#pragma unroll
        for (int d = 0; d < ND; d++) a[d] = f2d_bits(fm[d] * im);
    } else {
#pragma unroll
        for (int d = 0; d < ND; d++) a[d] = f[d] / m;
    }
    const double h = (MODE == DM_VERLET) ? P.dt_half : P.dtc2;
#pragma unroll
    for (int d = 0; d < ND; d++) v[d] = MIXED ? __fma_rn(a[d], h, v[d]) : v[d] + a[d] * h;
}

// Fused time-step kernel: [kick of the previous step] + drift of this step +
// FP32 position view + the neighbour-list displacement test (the reference
// runs that test at the end of the step; positions do not change after the
// drift, so testing here sees the same values).
template <int ND, int MODE, bool KICK, bool MIXED>
__global__ void __launch_bounds__(BLOCK) k_kickdrift(DevCtx c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    using V = typename DVec<ND>::T;
    bool valid = false;
    double dsq = 0.0;
    uint32_t s = i < c.n ? c.atom_sys[i] : 0u;
    if (i < c.n && c.active[s]) {
        const StepParams& P = *c.params;
        const double m = c.m[i];
        V xv = static_cast<V*>(c.x)[i];
        V vv = static_cast<V*>(c.v)[i];
        V av;
        double* x = reinterpret_cast<double*>(&xv);
        double* v = reinterpret_cast<double*>(&vv);
        double* a = reinterpret_cast<double*>(&av);
        const bool mob = MIXED ? mobile_bits(m) : mobile(m);
        if constexpr (MIXED && MODE == DM_VERLET) {
            // leapfrog form of the same update: the previous step's closing
            // half kick and this step's opening one use the same force, so
            // v_half += a dt and x += v_half dt (two FP64 fused
            // multiply-adds per axis instead of four)
#pragma unroll
            for (int d = 0; d < (int)(sizeof(V) / 8); d++) a[d] = 0.0;
            if (mob) {
                if constexpr (KICK) {
                    const float4 q = c.f32[i];
                    const float im = c.invm32[i];
                    a[0] = f2d_bits(q.x * im);
                    a[1] = f2d_bits(q.y * im);
                    if constexpr (ND == 3) a[2] = f2d_bits(q.z * im);
                } else {
                    av = static_cast<const V*>(c.a)[i];
                }
                const double hv = KICK ? P.dt : P.dt_half;
#pragma unroll
                for (int d = 0; d < ND; d++) {
                    v[d] = __fma_rn(a[d], hv, v[d]);
                    x[d] = __fma_rn(v[d], P.dt, x[d]);
                }
            } else {
#pragma unroll
                for (int d = 0; d < ND; d++) v[d] = 0.0;
            }
        } else {
        if constexpr (KICK) {
#pragma unroll
            for (int d = 0; d < (int)(sizeof(V) / 8); d++) a[d] = 0.0;
            kick<ND, MODE, MIXED>(c, i, m, a, v);
        } else {
            av = static_cast<const V*>(c.a)[i];
        }
        if (!mob) {
#pragma unroll
            for (int d = 0; d < ND; d++) v[d] = 0.0;
        } else if constexpr (MIXED && MODE != DM_SOL) {
            // the mixed path contracts the same FP64 updates into fused
            // multiply-adds (half the FP64 operations; it is not bit-exact)
            const double cv = MODE == DM_VERLET ? P.dt : P.c1dt;
            const double ca = MODE == DM_VERLET ? P.dt2_half : P.c2dtdt;
#pragma unroll
            for (int d = 0; d < ND; d++) {
                x[d] = __fma_rn(v[d], cv, __fma_rn(a[d], ca, x[d]));
                v[d] = MODE == DM_VERLET ? __fma_rn(a[d], P.dt_half, v[d])
                                         : __fma_rn(a[d], P.dtc12, v[d] * P.c0);
            }
        } else if constexpr (MODE == DM_VERLET) {
            // x += v*dt + a*(dt*dt/2); v += a*(dt/2)
#pragma unroll
            for (int d = 0; d < ND; d++) {
                x[d] = x[d] + (v[d] * P.dt + a[d] * P.dt2_half);
                v[d] = v[d] + a[d] * P.dt_half;
            }
        } else if constexpr (MODE == DM_DAMPED) {
            // x += v*(c1*dt) + a*(c2*dt*dt); v = v*c0 + a*(dt*(c1-c2))
#pragma unroll
            for (int d = 0; d < ND; d++) {
                x[d] = x[d] + (v[d] * P.c1dt + a[d] * P.c2dtdt);
                v[d] = v[d] * P.c0 + a[d] * P.dtc12;
            }
        } else {
            // CollectionSol: x += v*(c1*dt) + a*(c2*dt*dt) + drG*r0;
            //                v  = v*c0 + a*(dt*(c1-c2)) + dvG*v0
            double v0 = sqrt(P.T / m);
            double r0 = P.dt * v0;
            double g[6] = {0, 0, 0, 0, 0, 0};
            if (P.noise) normals6(c.seed[s], P.step, c.orig[i] - c.sys[s].atom_off, g);
#pragma unroll
            for (int d = 0; d < ND; d++) {
                double drG = g[d] * P.x11;
                double dvG = g[d] * P.x21 + g[ND + d] * P.x22;
                x[d] = x[d] + ((v[d] * P.c1dt + a[d] * P.c2dtdt) + drG * r0);
                v[d] = (v[d] * P.c0 + a[d] * P.dtc12) + dvG * v0;
            }
        }
        }
        if (mob) static_cast<V*>(c.x)[i] = xv;
        static_cast<V*>(c.v)[i] = vv;
        if (KICK && !MIXED) static_cast<V*>(c.a)[i] = av;
        if (mob) {
            // fine part of the FP32 position view against the coarse part fixed
            // at the last rebuild or upload (x - X is exact in FP64); an atom
            // that has moved more than 1/4 from its coarse point is re-anchored
            // (any multiple of 1/8 is a valid coarse point)
            // (mixed path: on the bit patterns, integer and FP32 instructions
            // only, within one ulp of (float)(x - X) and equal to it but for
            // rare roundings; FP64 path: the FP64 subtraction, exact, with the
            // conversions on the bit patterns)
            float4 A = c.pos[2 * (size_t)i];
            float4 B;
            auto fine = [](double xd, float Xf) {
                return MIXED ? fine_bits(xd, Xf) : d2f_bits(xd - f2d_bits(Xf));
            };
            B.x = fine(x[0], A.x);
            B.y = fine(x[1], A.y);
            B.z = 0.f;
            if constexpr (ND == 3) B.z = fine(x[2], A.z);
            B.w = 0.f;
            if (fabsf(B.x) > 0.25f || fabsf(B.y) > 0.25f || fabsf(B.z) > 0.25f) {
                posq_split2(x[0], A.x, B.x);
                posq_split2(x[1], A.y, B.y);
                if constexpr (ND == 3) posq_split2(x[2], A.z, B.z);
                c.pos[2 * (size_t)i] = A;
            }
            c.pos[2 * (size_t)i + 1] = B;
            if constexpr (MIXED)
                if (c.staged) c.rec[i] = make_record(A, B, c.rframe[i]);
        }
        if (c.rank[i] != NOT_MEMBER) {
            const V l = static_cast<const V*>(c.lastloc)[i];
            if constexpr (MIXED) {
                const double* lp = reinterpret_cast<const double*>(&l);
                const double d0 = x[0] - lp[0], d1 = x[1] - lp[1];
                dsq = __fma_rn(d1, d1, d0 * d0);
                if constexpr (ND == 3) {
                    const double d2 = x[2] - lp[2];
                    dsq = __fma_rn(d2, d2, dsq);
                }
            } else {
                dsq = disp_sq<ND>(xv, l);
            }
            // dsq is a sum of squares: +0, positive, +inf or NaN, so the tests
            // compare bit patterns (integer instructions, not the FP64 pipe)
            const unsigned long long db = (unsigned long long)__double_as_longlong(dsq);
            valid = (db & 0x7FFFFFFFFFFFFFFFull) <= 0x7FF0000000000000ull;
            // the cell-block records hold atoms within 2 skin + 1/2 of their
            // position at the last build (far more than the rebuild test lets
            // them move)
            if constexpr (MIXED)
                if (c.staged && valid &&
                    db > (unsigned long long)__double_as_longlong(c.sys[s].rec_lim2))
                    atomicOr(c.status, ST_IMAGE_RANGE);
        }
    }
    check_accumulate(c, s, valid, dsq);
}

// final kick of a call, so that the state between calls is the reference's
template <int ND, int MODE, bool MIXED>
__global__ void __launch_bounds__(BLOCK) k_kick(DevCtx c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n || !c.active[c.atom_sys[i]]) return;
    using V = typename DVec<ND>::T;
    V vv = static_cast<V*>(c.v)[i];
    V av;
    double* a = reinterpret_cast<double*>(&av);
#pragma unroll
    for (int d = 0; d < (int)(sizeof(V) / 8); d++) a[d] = 0.0;
    kick<ND, MODE, MIXED>(c, i, c.m[i], a, reinterpret_cast<double*>(&vv));
    static_cast<V*>(c.v)[i] = vv;
    static_cast<V*>(c.a)[i] = av;
}

template <int ND, int MODE, bool MIXED>
static void drift_nd(const DevCtx& c, cudaStream_t s, bool with_kick) {
    unsigned g = grid_for(c.n);
    if (with_kick) k_kickdrift<ND, MODE, true, MIXED><<<g, BLOCK, 0, s>>>(c);
    else k_kickdrift<ND, MODE, false, MIXED><<<g, BLOCK, 0, s>>>(c);
}

template <int ND, bool MIXED>
static void drift_prec(const DevCtx& c, cudaStream_t s, int mode, bool with_kick) {
    if (mode == DM_VERLET) drift_nd<ND, DM_VERLET, MIXED>(c, s, with_kick);
    else if (mode == DM_DAMPED) drift_nd<ND, DM_DAMPED, MIXED>(c, s, with_kick);
    else drift_nd<ND, DM_SOL, MIXED>(c, s, with_kick);
}

void launch_drift(const DevCtx& c, cudaStream_t s, int mode, bool with_kick) {
    if (c.nd == 3) {
        if (c.prec == PREC_MIXED) drift_prec<3, true>(c, s, mode, with_kick);
        else drift_prec<3, false>(c, s, mode, with_kick);
    } else {
        if (c.prec == PREC_MIXED) drift_prec<2, true>(c, s, mode, with_kick);
        else drift_prec<2, false>(c, s, mode, with_kick);
    }
}

template <int ND, bool MIXED>
static void kick_prec(const DevCtx& c, cudaStream_t s, int mode) {
    unsigned g = grid_for(c.n);
    if (mode == DM_VERLET) k_kick<ND, DM_VERLET, MIXED><<<g, BLOCK, 0, s>>>(c);
    else if (mode == DM_DAMPED) k_kick<ND, DM_DAMPED, MIXED><<<g, BLOCK, 0, s>>>(c);
    else k_kick<ND, DM_SOL, MIXED><<<g, BLOCK, 0, s>>>(c);
}

void launch_kick(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.nd == 3) {
        if (c.prec == PREC_MIXED) kick_prec<3, true>(c, s, mode);
        else kick_prec<3, false>(c, s, mode);
    } else {
        if (c.prec == PREC_MIXED) kick_prec<2, true>(c, s, mode);
        else kick_prec<2, false>(c, s, mode);
    }
}

// ---------------------------------------------------------------------------
// host AoS <-> internal SoA.  A record of caller atom o starts at
// staging + o*stride: x[0..nd), v[nd..2nd), a[2nd..3nd), f[3nd..4nd), m[4nd]
// (the reference's struct Atom {Vec x, v, a, f; flt m;}).
// ---------------------------------------------------------------------------
enum FieldBits : uint32_t { FB_X = 1, FB_V = 2, FB_A = 4, FB_F = 8, FB_M = 16 };

template <int ND>
__global__ void k_scatter_in(DevCtx c, const double* st, uint64_t stride, uint32_t fields) {
    uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= c.n) return;
    using V = typename DVec<ND>::T;
    uint32_t k = c.slot[o];
    const double* r = st + (uint64_t)o * stride;
    auto ld = [&](int off) {
        V t;
        double* p = reinterpret_cast<double*>(&t);
#pragma unroll
        for (int d = 0; d < (int)(sizeof(V) / 8); d++) p[d] = d < ND ? r[off + d] : 0.0;
        return t;
    };
    if (fields & FB_X) {
        V xv = ld(0);
        static_cast<V*>(c.x)[k] = xv;
        store_posq<ND>(c, k, reinterpret_cast<const double*>(&xv));
    }
    if (fields & FB_V) static_cast<V*>(c.v)[k] = ld(ND);
    if (fields & FB_A) static_cast<V*>(c.a)[k] = ld(2 * ND);
    if (fields & FB_F) {
        V fv = ld(3 * ND);
        static_cast<V*>(c.f)[k] = fv;
        const double* fp = reinterpret_cast<const double*>(&fv);
        c.f32[k] = make_float4((float)fp[0], (float)fp[1], ND == 3 ? (float)fp[ND - 1] : 0.f, 0.f);
    }
    if (fields & FB_M) {
        double m = r[4 * ND];
        c.m[k] = m;
        c.invm32[k] = mobile(m) ? (float)(1.0 / m) : 0.f;
        // a mass whose bits differ from the first record's
        if (__double_as_longlong(m) != __double_as_longlong(st[4 * ND])) atomicOr(c.m_mixed, 1u);
    }
}

template <int ND>
__global__ void k_gather_out(DevCtx c, double* st, uint64_t stride, uint32_t fields) {
    uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= c.n) return;
    using V = typename DVec<ND>::T;
    uint32_t k = c.slot[o];
    double* r = st + (uint64_t)o * stride;
    auto put = [&](int off, const V& t) {
        const double* p = reinterpret_cast<const double*>(&t);
#pragma unroll
        for (int d = 0; d < ND; d++) r[off + d] = p[d];
    };
    if (fields & FB_X) put(0, static_cast<const V*>(c.x)[k]);
    if (fields & FB_V) put(ND, static_cast<const V*>(c.v)[k]);
    if (fields & FB_A) put(2 * ND, static_cast<const V*>(c.a)[k]);
    if (fields & FB_F) {
        if (c.prec == PREC_MIXED) {
            float4 f = c.f32[k];
            r[3 * ND] = f.x;
            r[3 * ND + 1] = f.y;
            if (ND == 3) r[3 * ND + ND - 1] = f.z;
        } else {
            put(3 * ND, static_cast<const V*>(c.f)[k]);
        }
    }
    if (fields & FB_M) r[4 * ND] = c.m[k];
}

void launch_scatter_in(const DevCtx& c, cudaStream_t s, const double* st, uint64_t stride,
                       uint32_t fields) {
    if (fields & FB_M) cudaMemsetAsync(c.m_mixed, 0, sizeof(uint32_t), s);   // every mass is uploaded
    if (c.nd == 3) k_scatter_in<3><<<grid_for(c.n), BLOCK, 0, s>>>(c, st, stride, fields);
    else k_scatter_in<2><<<grid_for(c.n), BLOCK, 0, s>>>(c, st, stride, fields);
}

void launch_gather_out(const DevCtx& c, cudaStream_t s, double* st, uint64_t stride,
                       uint32_t fields) {
    if (c.nd == 3) k_gather_out<3><<<grid_for(c.n), BLOCK, 0, s>>>(c, st, stride, fields);
    else k_gather_out<2><<<grid_for(c.n), BLOCK, 0, s>>>(c, st, stride, fields);
}

// ---------------------------------------------------------------------------
// per-atom reduction inputs (component-major: red[comp * n + i])
// ---------------------------------------------------------------------------
template <int ND>
__global__ void k_atoms(DevCtx c, int what, const double* origin) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    using V = typename DVec<ND>::T;
    double m = c.m[i];
    uint32_t s = c.atom_sys[i];
    if (what == AW_KINETIC) {
        // AtomGroup::kinetic_energy (box.cpp:401-411): skip m == 0 or inf
        double e = 0.0;
        if (!(m == 0.0 || isinf(m))) {
            V vv = static_cast<const V*>(c.v)[i];
            const double* v = reinterpret_cast<const double*>(&vv);
            double cv[3] = {0, 0, 0};
#pragma unroll
            for (int d = 0; d < ND; d++) cv[d] = v[d] - (origin ? origin[s * ND + d] : 0.0);
            double dd = cv[0] * cv[0] + cv[1] * cv[1];
            if constexpr (ND == 3) dd = dd + cv[2] * cv[2];
            e = m / 2 * dd;
        }
        c.red[i] = e;
    } else if (what == AW_MOMENTUM) {
        // AtomGroup::momentum / mass (box.cpp:237-258): skip m <= 0 or inf
        bool ok = mobile(m);
        V vv = static_cast<const V*>(c.v)[i];
        const double* v = reinterpret_cast<const double*>(&vv);
#pragma unroll
        for (int d = 0; d < ND; d++) c.red[(size_t)d * c.n + i] = ok ? v[d] * m : 0.0;
        c.red[(size_t)ND * c.n + i] = ok ? m : 0.0;
    } else if (what == AW_COM) {
        // AtomGroup::com / mass (box.cpp:228-247): skip m <= 0 or inf
        bool ok = mobile(m);
        V xv = static_cast<const V*>(c.x)[i];
        const double* x = reinterpret_cast<const double*>(&xv);
#pragma unroll
        for (int d = 0; d < ND; d++) c.red[(size_t)d * c.n + i] = ok ? x[d] * m : 0.0;
        c.red[(size_t)ND * c.n + i] = ok ? m : 0.0;
    } else {
        double q = 0.0;
        if (mobile(m)) {
            if (c.prec == PREC_MIXED) {
                float4 f = c.f32[i];
                q = (double)f.x * f.x + (double)f.y * f.y + (double)f.z * f.z;
            } else {
                V fv = static_cast<const V*>(c.f)[i];
                const double* f = reinterpret_cast<const double*>(&fv);
                q = f[0] * f[0] + f[1] * f[1];
                if constexpr (ND == 3) q = q + f[2] * f[2];
            }
        }
        c.red[i] = q;
    }
}

void launch_reduce_atoms(const DevCtx& c, cudaStream_t s, int what, const double* origin) {
    if (c.nd == 3) k_atoms<3><<<grid_for(c.n), BLOCK, 0, s>>>(c, what, origin);
    else k_atoms<2><<<grid_for(c.n), BLOCK, 0, s>>>(c, what, origin);
}

// Deterministic per-system reduction of red[comp * n + i] over each system's
// atoms in two passes with a fixed order: every chunk of up to RED_CHUNK
// consecutive atoms of one system is reduced by one CTA (fixed striding and
// tree), then one CTA per system reduces its chunks in chunk order.  ncomp < 0
// means a single-component maximum.
template <int NT>
__device__ __forceinline__ double block_reduce(double acc, bool is_max, double* sh) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_down_sync(0xFFFFFFFFu, acc, off);
        acc = is_max ? fmax(acc, o) : acc + o;
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    double v = 0.0;
    if (threadIdx.x < 32) {
        v = threadIdx.x < NT / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double o = __shfl_down_sync(0xFFFFFFFFu, v, off);
            v = is_max ? fmax(v, o) : v + o;
        }
    }
    __syncthreads();
    return v;   // valid in thread 0
}

constexpr int RED_THREADS = 256;

__global__ void __launch_bounds__(RED_THREADS) k_red_chunks(DevCtx c, int ncomp) {
    __shared__ double sh[32];
    const uint4 ch = c.chunk[blockIdx.x];   // (system, first atom, atoms, -)
    const bool is_max = ncomp < 0;
    const int nc = is_max ? 1 : ncomp;
    for (int comp = 0; comp < nc; comp++) {
        const double* r = c.red + (size_t)comp * c.n + ch.y;
        double acc = 0.0;
        for (uint32_t k = threadIdx.x; k < ch.z; k += RED_THREADS) {
            const double v = r[k];
            acc = is_max ? fmax(acc, v) : acc + v;
        }
        acc = block_reduce<RED_THREADS>(acc, is_max, sh);
        if (threadIdx.x == 0) c.part[(size_t)blockIdx.x * nc + comp] = acc;
    }
}

__global__ void __launch_bounds__(RED_THREADS) k_sys_reduce(DevCtx c, int ncomp) {
    __shared__ double sh[32];
    const uint32_t s = blockIdx.x;
    const bool is_max = ncomp < 0;
    const int nc = is_max ? 1 : ncomp;
    const uint32_t k0 = c.sys_chunk[s], k1 = c.sys_chunk[s + 1];
    for (int comp = 0; comp < nc; comp++) {
        double acc = 0.0;
        for (uint32_t k = k0 + threadIdx.x; k < k1; k += RED_THREADS) {
            const double v = c.part[(size_t)k * nc + comp];
            acc = is_max ? fmax(acc, v) : acc + v;
        }
        acc = block_reduce<RED_THREADS>(acc, is_max, sh);
        if (threadIdx.x == 0) c.sysout[(size_t)s * nc + comp] = acc;
    }
}

void launch_sys_reduce(const DevCtx& c, cudaStream_t s, int ncomp) {
    k_red_chunks<<<c.nchunk, RED_THREADS, 0, s>>>(c, ncomp);
    k_sys_reduce<<<c.nsys, RED_THREADS, 0, s>>>(c, ncomp);
}

// ---------------------------------------------------------------------------
// Mean-square-displacement tracker: RsqTracker / RsqTracker1
// (src/constraints.hpp:318-361, src/constraints.cpp:404-560).  Per atom (by
// caller index) and window j: the position r = x - com at the window's last
// update and the running sums of (r - r_past)^2 per axis, of its square, and
// of the squared squared distance.  One update advances the tracker time t
// and updates the windows whose length divides t, in the reference's
// arithmetic (componentwise FP64, no contraction).
// ---------------------------------------------------------------------------
// the update's preamble: the tracker time (thread 0; not at the start) and
// each system's centre of mass, (sum of m x) / mass per axis as
// AtomGroup::com (one thread per system)
__global__ void k_rsq_prep(DevCtx c, int init) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0 && !init) {
        const unsigned long long t = c.rsq_cnt[0] + 1ull;
        c.rsq_cnt[0] = t;
        for (uint32_t j = 0; j < c.rsq_n; j++)
            if (t % c.rsq_skip[j] == 0ull) c.rsq_cnt[1 + j] += 1ull;
    }
    if (s >= c.nsys) return;
    const int nd = c.nd;
    for (int d = 0; d < nd; d++)
        c.rsq_comv[(size_t)s * 3 + d] =
            c.rsq_com ? c.sysout[(size_t)s * (nd + 1) + d] / c.sysout[(size_t)s * (nd + 1) + nd] : 0.0;
}

// one thread per atom in caller order (the tracker's arrays are read and
// written in order; the position is gathered through the atom's slot)
template <int ND, bool INIT>
__global__ void k_rsq(DevCtx c) {
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= c.n) return;
    using V = typename DVec<ND>::T;
    const uint32_t i = c.slot[o], s = c.atom_sys[i];
    V xv = static_cast<const V*>(c.x)[i];
    const double* x = reinterpret_cast<const double*>(&xv);
    double r[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < ND; d++) r[d] = x[d] - c.rsq_comv[(size_t)s * 3 + d];   // zero without com
    const unsigned long long t = c.rsq_cnt[0];
    for (uint32_t j = 0; j < c.rsq_n; j++) {
        const size_t base = ((size_t)j * c.n + o) * ND;
        if (INIT) {
#pragma unroll
            for (int d = 0; d < ND; d++) c.rsq_past[base + d] = r[d];
            continue;
        }
        if (t % c.rsq_skip[j] != 0ull) continue;
        double ds[3], d4[3];
        double dist4 = 0.0;
#pragma unroll
        for (int d = 0; d < ND; d++) {
            ds[d] = r[d] - c.rsq_past[base + d];
            ds[d] = ds[d] * ds[d];
            d4[d] = ds[d] * ds[d];
            dist4 = dist4 + ds[d];
        }
        dist4 = dist4 * dist4;
#pragma unroll
        for (int d = 0; d < ND; d++) {
            c.rsq_x2[base + d] = c.rsq_x2[base + d] + ds[d];
            c.rsq_x4[base + d] = c.rsq_x4[base + d] + d4[d];
            c.rsq_past[base + d] = r[d];
        }
        c.rsq_r4[(size_t)j * c.n + o] = c.rsq_r4[(size_t)j * c.n + o] + dist4;
    }
}

void launch_rsq(const DevCtx& c, cudaStream_t s, int init) {
    if (!c.rsq_n) return;
    if (c.rsq_com) {
        launch_reduce_atoms(c, s, AW_COM, nullptr);
        launch_sys_reduce(c, s, c.nd + 1);
    }
    k_rsq_prep<<<(c.nsys + 255) / 256, 256, 0, s>>>(c, init);
    if (c.nd == 3) {
        if (init) k_rsq<3, true><<<grid_for(c.n), BLOCK, 0, s>>>(c);
        else k_rsq<3, false><<<grid_for(c.n), BLOCK, 0, s>>>(c);
    } else {
        if (init) k_rsq<2, true><<<grid_for(c.n), BLOCK, 0, s>>>(c);
        else k_rsq<2, false><<<grid_for(c.n), BLOCK, 0, s>>>(c);
    }
}

// ---- test hooks of the Langevin generator (parm_debug_philox / parm_debug_normals) ----
// in: 6 words per item (counter c0..c3, key k0, k1); out: the 4 output words
__global__ void k_philox_test(const uint32_t* in, uint32_t* out, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c[4] = {in[6 * (size_t)i], in[6 * (size_t)i + 1], in[6 * (size_t)i + 2], in[6 * (size_t)i + 3]};
    philox10(c, in[6 * (size_t)i + 4], in[6 * (size_t)i + 5]);
#pragma unroll
    for (int q = 0; q < 4; q++) out[4 * (size_t)i + q] = c[q];
}

// the six normals the Langevin step draws for atoms 0..n-1 of a system keyed `key` at counter `step`
__global__ void k_normals_test(unsigned long long key, unsigned long long step, uint32_t n, double* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double g[6];
    normals6(key, step, i, g);
#pragma unroll
    for (int q = 0; q < 6; q++) out[6 * (size_t)i + q] = g[q];
}

// the bit-pattern conversions of the per-atom update on n values of each kind
__global__ void k_fpbits_test(const double* d, const float* f, uint32_t n, float* d2f, double* f2d) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d2f[i] = d2f_bits(d[i]);
    f2d[i] = f2d_bits(f[i]);
}

void launch_fpbits_test(const double* d, const float* f, uint32_t n, float* d2f, double* f2d, cudaStream_t s) {
    if (n) k_fpbits_test<<<grid_for(n), BLOCK, 0, s>>>(d, f, n, d2f, f2d);
}

void launch_philox_test(const uint32_t* in, uint32_t* out, uint32_t n, cudaStream_t s) {
    if (n) k_philox_test<<<grid_for(n), BLOCK, 0, s>>>(in, out, n);
}

void launch_normals_test(unsigned long long key, unsigned long long step, uint32_t n, double* out,
                         cudaStream_t s) {
    if (n) k_normals_test<<<grid_for(n), BLOCK, 0, s>>>(key, step, n, out);
}

}  // namespace parm
