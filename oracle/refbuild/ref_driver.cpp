// Fixture driver: runs the reference's own classes (built from its sources
// by oracle/refbuild/Makefile) on an input deck and prints every quantity the
// parity tests compare, with 17 significant digits.  Test infrastructure.
//
// Input (whitespace separated): kind integrator nsteps dt damping T skin
//   L[NDIM] [gamma: kinds 100 + k, a LeesEdwardsBox of shear gamma]  N  then per atom x[NDIM] v[NDIM] m p0 p1 p2 (and p3 for kinds 4-7)
//   norder order[norder]   nign (a b)[nign]   nout out_steps[nout]
//   integrators 3 and 4 add one line: dt P0 kappa kmax secmax seceps alphamax afrac
//   dxmax stepmax maxdV
// kind: 0 NListed<EpsSigCutAtom,LennardJonesCutPair>, 1 <EpsSigExpAtom,RepulsionPair>,
//       2 <EpsSigAtom,LJRepulsePair>, 3 <EpsSigCutAtom,LJAttractCutPair>,
//       4 <LoisOhernAtom,LoisOhernPair>, 5 <LoisOhernAtom,LoisOhernPairMinCLs> (p: eps sigma C l),
//       6 <LoisLinAtom,LoisLinPair>, 7 <LoisLinAtom,LoisLinPairMin> (p: eps sigma depth width),
//       8 <EisMclachlanAtom,EisMclachlanPair> (p: dist sigmai unused),
//       9 <EpsSigExpDragAtom,RepulsionDragPair> (p: eps sigma gamma exponent),
//       indexed epsilons (the deck adds "nt eps[nt*nt] sig[nt*nt]" after the atoms; an atom of
//       type t gets row t): 10 <IEpsISigCutAtom,LennardJonesCutPair> (p: t sigcut unused),
//       11 <IEpsISigCutAtom,LJAttractCutPair> (same), 12 <IEpsSigCutAtom,LJAttractCutPair>
//       (p: t sigma sigcut), 13 <IEpsSigCutAtom,LJAttractRepulsePair> (same),
//       14 <IEpsRepsSigCutAtom,LJAttractFixedRepulsePair> (p: t repeps sigma sigcut),
//       15 <IEpsRepsSigExpCutAtom,LJishPair> (p: t repeps sigma n sigcut),
//       16 <IEpsISigExpAtom,RepulsionPair> (p: t exponent unused),
//       17 <EpsEpsSigSigCutAtom,LJAttractRepulseSigsPair> (p: eps_r eps_a sig_r sig_a sigcut);
//       integrator: 0 Verlet, 1 Damped, 2 Sol (T = 0),
//       3 CollectionNLCG (set up as pyparm's packmin.Minimizer does: constructor,
//       set_max_alpha / set_max_dx / set_max_step, set_forces(true, true)),
//       4 CollectionNLCGV (constructor, then reset())
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "collection.hpp"
#include "interaction.hpp"

// numbers are read with strtod so that "inf" and "nan" parse like any value
static double rd() {
    std::string t;
    if (!(std::cin >> t)) {
        std::fprintf(stderr, "ref_driver: truncated input\n");
        std::exit(2);
    }
    return std::strtod(t.c_str(), nullptr);
}
static unsigned rdu() { return (unsigned)rd(); }

static void pvec(const Vec& v) {
    for (int d = 0; d < NDIM; d++) std::printf(" %.17g", v[d]);
}

// a LeesEdwardsBox instead of the OriginBox (kinds 100 + k)
static bool g_lees = false;

// the pair tables of the indexed kinds
static unsigned g_nt = 0;
static std::vector<double> g_eps, g_sig;
static std::vector<flt> row_of(const std::vector<double>& t, unsigned r) {
    return std::vector<flt>(t.begin() + (size_t)r * g_nt, t.begin() + (size_t)(r + 1) * g_nt);
}

template <class A>
A make_atom(AtomID id, int kind, const double* p);
template <>
EpsSigCutAtom make_atom<EpsSigCutAtom>(AtomID id, int, const double* p) {
    return EpsSigCutAtom(id, p[0], p[1], p[2]);
}
template <>
EpsSigExpAtom make_atom<EpsSigExpAtom>(AtomID id, int, const double* p) {
    return EpsSigExpAtom(id, p[0], p[1], p[2]);
}
template <>
EpsSigAtom make_atom<EpsSigAtom>(AtomID id, int, const double* p) {
    return EpsSigAtom(id, p[0], p[1]);
}
template <>
LoisOhernAtom make_atom<LoisOhernAtom>(AtomID id, int, const double* p) {
    return LoisOhernAtom(id, p[0], p[1], p[2], p[3]);
}
template <>
LoisLinAtom make_atom<LoisLinAtom>(AtomID id, int, const double* p) {
    return LoisLinAtom(id, p[0], p[1], p[2], p[3]);
}
template <>
EisMclachlanAtom make_atom<EisMclachlanAtom>(AtomID id, int, const double* p) {
    return EisMclachlanAtom(id, p[0], p[1]);
}
template <>
EpsSigExpDragAtom make_atom<EpsSigExpDragAtom>(AtomID id, int, const double* p) {
    return EpsSigExpDragAtom(id, p[0], p[1], p[2], p[3]);
}
template <>
IEpsISigCutAtom make_atom<IEpsISigCutAtom>(AtomID id, int, const double* p) {
    const unsigned t = (unsigned)p[0];
    return IEpsISigCutAtom(id, row_of(g_eps, t), row_of(g_sig, t), t, p[1]);
}
template <>
IEpsSigCutAtom make_atom<IEpsSigCutAtom>(AtomID id, int, const double* p) {
    const unsigned t = (unsigned)p[0];
    return IEpsSigCutAtom(id, row_of(g_eps, t), t, p[1], p[2]);
}
template <>
IEpsRepsSigCutAtom make_atom<IEpsRepsSigCutAtom>(AtomID id, int, const double* p) {
    const unsigned t = (unsigned)p[0];
    return IEpsRepsSigCutAtom(id, row_of(g_eps, t), p[1], p[2], t, p[3]);
}
template <>
EpsEpsSigSigCutAtom make_atom<EpsEpsSigSigCutAtom>(AtomID id, int, const double* p) {
    return EpsEpsSigSigCutAtom(id, p[0], p[1], p[2], p[3], p[4]);
}
template <>
IEpsISigExpAtom make_atom<IEpsISigExpAtom>(AtomID id, int, const double* p) {
    const unsigned t = (unsigned)p[0];
    return IEpsISigExpAtom(id, row_of(g_eps, t), row_of(g_sig, t), t, p[1]);
}
template <>
IEpsRepsSigExpCutAtom make_atom<IEpsRepsSigExpCutAtom>(AtomID id, int, const double* p) {
    const unsigned t = (unsigned)p[0];
    return IEpsRepsSigExpCutAtom(id, row_of(g_eps, t), p[1], p[2], p[3], t, p[4]);
}

template <class A, class P>
int run(int kind, int integ, int nsteps, double dt, double damping, double T, double skin) {
    Vec L;
    for (int d = 0; d < NDIM; d++) L[d] = rd();
    const bool lees = g_lees;
    const double gamma = lees ? rd() : 0.0;
    unsigned N = rdu();
    const unsigned np = ((kind >= 4 && kind <= 7) || kind == 9 || kind == 14) ? 4 : ((kind == 15 || kind == 17) ? 5 : 3);
    std::vector<double> xs(N * NDIM), vs(N * NDIM), ms(N), ps(N * np);
    for (unsigned i = 0; i < N; i++) {
        for (int d = 0; d < NDIM; d++) xs[i * NDIM + d] = rd();
        for (int d = 0; d < NDIM; d++) vs[i * NDIM + d] = rd();
        ms[i] = rd();
        for (unsigned k = 0; k < np; k++) ps[np * i + k] = rd();
    }
    if (kind >= 10 && kind <= 16) {
        g_nt = rdu();
        g_eps.resize((size_t)g_nt * g_nt);
        g_sig.resize((size_t)g_nt * g_nt);
        for (auto& q : g_eps) q = rd();
        for (auto& q : g_sig) q = rd();
    }
    std::vector<unsigned> order(rdu());
    for (auto& o : order) o = rdu();
    std::vector<unsigned> ign(2 * rdu());
    for (auto& q : ign) q = rdu();
    std::vector<int> outs(rdu());
    for (auto& q : outs) q = (int)rd();
    double cg[11] = {0};
    if (integ >= 3)
        for (double& q : cg) q = rd();

    boost::shared_ptr<OriginBox> obox(lees ? new LeesEdwardsBox(L, gamma) : new OriginBox(L));
    boost::shared_ptr<AtomVec> atoms(new AtomVec(ms));
    for (unsigned i = 0; i < N; i++) {
        for (int d = 0; d < NDIM; d++) {
            (*atoms)[i].x[d] = xs[i * NDIM + d];
            (*atoms)[i].v[d] = vs[i * NDIM + d];
        }
    }
    boost::shared_ptr<NListed<A, P> > inter(new NListed<A, P>(obox, atoms, skin));
    boost::shared_ptr<NeighborList> nl = inter->neighbor_list();
    for (unsigned i : order) inter->add(make_atom<A>(atoms->get_id(i), kind, &ps[np * i]));
    for (size_t q = 0; q < ign.size() / 2; q++) nl->ignore(atoms->get_id(ign[2 * q]), atoms->get_id(ign[2 * q + 1]));
    nl->update_list(true);
    std::printf("PAIRS %u\n", nl->numpairs());
    for (unsigned k = 0; k < nl->numpairs(); k++) {
        IDPair pr = nl->get(k);
        std::printf("%u %u\n", pr.first().n(), pr.last().n());
    }

    std::vector<boost::shared_ptr<Interaction> > is(1, inter);
    std::vector<boost::shared_ptr<StateTracker> > ts(1, nl);
    boost::shared_ptr<Collection> col;
    boost::shared_ptr<CollectionNLCG> cg3;
    boost::shared_ptr<CollectionNLCGV> cg4;
    std::vector<boost::shared_ptr<Constraint> > cs;
    if (integ == 0) col.reset(new CollectionVerlet(obox, atoms, dt, is, ts));
    else if (integ == 1) col.reset(new CollectionDamped(obox, atoms, dt, damping, is, ts));
    else if (integ == 2) col.reset(new CollectionSol(obox, atoms, dt, damping, T, is, ts));
    else if (integ == 3) {
        cg3.reset(new CollectionNLCG(obox, atoms, cg[0], cg[1], is, ts, cs, cg[2], cg[3], (uint)cg[4], cg[5]));
        cg3->set_max_alpha(cg[6]);
        cg3->set_max_alpha_fraction(cg[7]);
        cg3->set_max_dx(cg[8]);
        cg3->set_max_step(cg[9]);
        cg3->maxdV = cg[10];
        cg3->set_forces(true, true);
        col = cg3;
    } else {
        cg4.reset(new CollectionNLCGV(obox, atoms, cg[0], is, ts, cs, cg[3], (uint)cg[4], cg[5]));
        cg4->set_max_alpha(cg[6]);
        cg4->set_max_alpha_fraction(cg[7]);
        cg4->set_max_dx(cg[8]);
        cg4->set_max_step(cg[9]);
        cg4->reset();
        col = cg4;
    }

    Matrix st = inter->stress(*obox);
    std::printf("INIT %.17g %.17g %llu %llu %u\n", inter->energy(*obox), inter->pressure(*obox),
                inter->contacts(*obox), inter->overlaps(*obox), nl->which());
    for (int a = 0; a < NDIM; a++)
        for (int b = 0; b < NDIM; b++) std::printf(" %.17g", st(a, b));
    std::printf("\n");
    for (unsigned i = 0; i < N; i++) {
        pvec((*atoms)[i].f);
        pvec((*atoms)[i].a);
        std::printf("\n");
    }
    int step = 0;
    for (int target : outs) {
        while (step < target && step < nsteps) {
            col->timestep();
            step++;
        }
        std::printf("STEP %d %u %.17g %.17g\n", step, nl->which(), inter->energy(*obox), atoms->kinetic_energy());
        if (integ >= 3) {
            const Vec Lb = obox->box_shape();
            std::printf("NLCG");
            pvec(Lb);
            if (cg3)
                std::printf(" %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %u\n", cg3->Knew, cg3->k,
                            cg3->vl, cg3->fl, cg3->al, cg3->alpha, cg3->beta, cg3->betaused, cg3->dxsum,
                            cg3->alphavmax, cg3->sec);
            else
                std::printf(" %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %u\n", cg4->Knew, cg4->k,
                            cg4->vl, cg4->fl, cg4->al, cg4->alpha, cg4->beta, cg4->betaused, cg4->dxsum,
                            cg4->alphavmax, cg4->sec);
        }
        for (unsigned i = 0; i < N; i++) {
            pvec((*atoms)[i].x);
            pvec((*atoms)[i].v);
            pvec((*atoms)[i].a);
            pvec((*atoms)[i].f);
            std::printf("\n");
        }
    }
    return 0;
}

int main() {
    int kind = (int)rd(), integ = (int)rd(), nsteps = (int)rd();
    if (kind >= 100) {
        g_lees = true;
        kind -= 100;
    }
    double dt = rd(), damping = rd(), T = rd(), skin = rd();
    if (kind == 0) return run<EpsSigCutAtom, LennardJonesCutPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 1) return run<EpsSigExpAtom, RepulsionPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 3) return run<EpsSigCutAtom, LJAttractCutPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 4) return run<LoisOhernAtom, LoisOhernPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 5) return run<LoisOhernAtom, LoisOhernPairMinCLs>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 6) return run<LoisLinAtom, LoisLinPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 7) return run<LoisLinAtom, LoisLinPairMin>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 8) return run<EisMclachlanAtom, EisMclachlanPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 9) return run<EpsSigExpDragAtom, RepulsionDragPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 10) return run<IEpsISigCutAtom, LennardJonesCutPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 11) return run<IEpsISigCutAtom, LJAttractCutPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 12) return run<IEpsSigCutAtom, LJAttractCutPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 13) return run<IEpsSigCutAtom, LJAttractRepulsePair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 14)
        return run<IEpsRepsSigCutAtom, LJAttractFixedRepulsePair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 15) return run<IEpsRepsSigExpCutAtom, LJishPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 16) return run<IEpsISigExpAtom, RepulsionPair>(kind, integ, nsteps, dt, damping, T, skin);
    if (kind == 17)
        return run<EpsEpsSigSigCutAtom, LJAttractRepulseSigsPair>(kind, integ, nsteps, dt, damping, T, skin);
    return run<EpsSigAtom, LJRepulsePair>(kind, integ, nsteps, dt, damping, T, skin);
}
