// parm_gb300 host API implementation: the reference's C++ classes
// (wackywendell/parm src/box.*, src/trackers.*, src/interaction.hpp,
// src/collection.*) on top of the C ABI of include/parm_gb300.h.
#include <algorithm>
#include <cstdlib>
#include <functional>
#include <cstring>
#include <stdexcept>
#include <string>

#include "collection.hpp"

// ---------------------------------------------------------------------------
// random numbers (std::mt19937; the reference's vecrand.cpp uses Boost's)
std::mt19937& parm_random_engine() {
    static std::mt19937 eng(5489u);
    return eng;
}
flt rand01() { return std::uniform_real_distribution<flt>(0.0, 1.0)(parm_random_engine()); }
Vec rand_vec() {
    std::normal_distribution<flt> g(0.0, 1.0);
    Vec v;
    for (int d = 0; d < NDIM; d++) v[d] = g(parm_random_engine());
    return v;
}
Vec rand_vec_boxed() {
    Vec v;
    for (int d = 0; d < NDIM; d++) v[d] = rand01();
    return v;
}
unsigned int seed(unsigned int n) {
    parm_random_engine().seed(n);
    return n;
}
unsigned int seed() { return seed(static_cast<unsigned int>(time(nullptr))); }

// ---------------------------------------------------------------------------
// AtomGroup (src/box.cpp:237-258, 395-415)
flt AtomGroup::mass() const {
    flt m = 0;
    for (uint i = 0; i < size(); i++) {
        const Atom& a = (*this)[i];
        if (a.m <= 0 || std::isinf(a.m)) continue;
        m += a.m;
    }
    return m;
}

Vec AtomGroup::momentum() const {
    Vec tot = Vec::Zero();
    for (uint i = 0; i < size(); i++) {
        const Atom& a = (*this)[i];
        if (a.m <= 0 || std::isinf(a.m)) continue;
        tot += a.v * a.m;
    }
    return tot;
}

flt AtomGroup::kinetic_energy(const Vec originvelocity) const {
    flt totE = 0;
    for (uint i = 0; i < size(); i++) {
        const Atom& a = (*this)[i];
        if (a.m == 0 || std::isinf(a.m)) continue;
        const Vec curv = a.v - originvelocity;
        totE += a.m / 2 * curv.dot(curv);
    }
    return totE;
}

void AtomGroup::add_velocity(Vec v) {
    for (uint i = 0; i < size(); i++) (*this)[i].v += v;
}

void AtomGroup::reset_forces() {
    for (uint i = 0; i < size(); i++) (*this)[i].f = Vec::Zero();
}

void AtomGroup::randomize_velocities(flt T) {
    // src/box.cpp:419-425: atoms of zero or infinite mass keep their velocity
    for (uint i = 0; i < size(); i++) {
        Atom& a = (*this)[i];
        if (a.m == 0 || std::isinf(a.m)) continue;
        a.v = rand_vec() * std::sqrt(T / a.m);
    }
}

flt OriginBox::resize(flt factor, AtomGroup& atoms) {
    boxsize *= factor;
    for (uint i = 0; i < atoms.size(); i++) atoms[i].x *= factor;
    return V();
}

// LeesEdwardsBox::shear / shear_to with the atoms (src/box.cpp:103-135):
// x += y * dgamma
void LeesEdwardsBox::shear(flt dgamma, AtomGroup& atoms) {
    for (uint i = 0; i < atoms.size(); i++) {
        const flt dy = atoms[i].x[1];
        atoms[i].x[0] += dy * dgamma;
    }
    gamma += dgamma;
}

void LeesEdwardsBox::shear_to(flt new_gamma, AtomGroup& atoms) {
    for (uint i = 0; i < atoms.size(); i++) {
        const flt dy = atoms[i].x[1];
        atoms[i].x[0] += dy * (new_gamma - gamma);
    }
    gamma = new_gamma;
}

flt OriginBox::resize_to(Vec newsize, AtomGroup& atoms) {
    const Vec scale = newsize.cwiseQuotient(boxsize);
    boxsize = newsize;
    for (uint i = 0; i < atoms.size(); i++) atoms[i].x = atoms[i].x.cwiseProduct(scale);
    return V();
}

// ---------------------------------------------------------------------------
// GPU handles
static int g_precision = -1;

void parm_host_set_precision(int precision) { g_precision = precision; }

int parm_host_precision() {
    if (g_precision < 0) {
        const char* e = std::getenv("PARM_PRECISION");
        g_precision = (e && std::strcmp(e, "mixed") == 0) ? PARM_MIXED : PARM_FP64;
    }
    return g_precision;
}

void parm_host_check(int rc, const char* what) {
    if (rc != PARM_OK) throw std::runtime_error(std::string(what) + ": " + parm_last_error());
}

GpuLink::GpuLink(sptr<Box> box, sptr<AtomVec> atoms, flt skin) : bx(box), atomv(atoms), skin_(skin) {
    if (!std::dynamic_pointer_cast<OriginBox>(bx))
        throw std::invalid_argument("parm_gb300: the GPU path supports periodic OriginBox boxes");
    params.assign(5 * (size_t)atomv->size(), 0.0);
    rank.assign(atomv->size(), PARM_NOT_MEMBER);
    ldiam.assign(atomv->size(), std::nan(""));
}

GpuLink::~GpuLink() {
    if (h) parm_destroy(h);
}

void GpuLink::add(uint atom, int k, const double p[5], const void* owner) {
    if (atom >= atomv->size()) throw std::out_of_range("NListed::add: atom not in this AtomVec");
    if (owner_ && owner != owner_)
        throw std::invalid_argument("parm_gb300: one NListed interaction per NeighborList");
    if (kind >= 0 && k != kind) throw std::invalid_argument("NListed::add: one pair law per interaction");
    if (rank[atom] != PARM_NOT_MEMBER) throw std::invalid_argument("NListed::add: atom added twice");
    owner_ = owner;
    kind = k;
    for (int q = 0; q < PARM_NPARAM(k); q++) params[5 * (size_t)atom + q] = p[q];
    rank[atom] = nmembers++;
    interaction_dirty = true;
}

void GpuLink::set_type_row(uint type, const std::vector<flt>& eps, const std::vector<flt>* sig) {
    if (type >= eps.size()) throw std::invalid_argument("NListed::add: the atom's index is not in its epsilons");
    std::vector<double> e(eps.begin(), eps.end());
    std::vector<double> sg;
    if (sig) sg.assign(sig->begin(), sig->end());
    if (type >= eps_rows.size()) {
        eps_rows.resize(type + 1);
        sig_rows.resize(type + 1);
    }
    if (!eps_rows[type].empty()) {
        if (eps_rows[type] != e || sig_rows[type] != sg)
            throw std::invalid_argument("parm_gb300: atoms of one type index must share their epsilons and sigmas");
        return;
    }
    eps_rows[type] = e;
    sig_rows[type] = sg;
    rows_dirty = true;
}

void GpuLink::add_member(uint atom, double diameter) {
    if (atom >= atomv->size()) throw std::out_of_range("NeighborList::add: atom not in this AtomVec");
    if (rank[atom] != PARM_NOT_MEMBER) throw std::invalid_argument("NeighborList::add: atom added twice");
    if (!(diameter >= 0.0)) throw std::invalid_argument("NeighborList::add: diameter must be >= 0");
    rank[atom] = nmembers++;
    ldiam[atom] = diameter;
    any_ldiam = true;
    interaction_dirty = true;
}

void GpuLink::ignore(uint a, uint b) {
    pending_ignores.emplace_back(a, b);
    nignored++;
}

void GpuLink::push() {
    if (!h) {
        uint32_t n = atomv->size();
        parm_host_check(parm_create(&h, NDIM, 1, &n, parm_host_precision()), "parm_create");
    }
    OriginBox& ob = *std::dynamic_pointer_cast<OriginBox>(bx);
    const Vec L = ob.box_shape();
    std::vector<double> lv(L.data(), L.data() + NDIM);
    if (lv != lastbox) {
        parm_host_check(parm_set_boxes(h, lv.data()), "parm_set_boxes");
        lastbox = lv;
    }
    if (auto le = std::dynamic_pointer_cast<LeesEdwardsBox>(bx)) {
        const double g = le->get_gamma();
        if (!(g == lastgamma)) {
            parm_host_check(parm_set_lees_edwards(h, &g), "parm_set_lees_edwards");
            lastgamma = g;
        }
    }
    if (rows_dirty) {
        // the table of the indexed kinds: row a = the epsilons of the atoms of type a
        size_t nt = eps_rows.size();
        for (auto& r : eps_rows) nt = std::max(nt, r.size());
        std::vector<double> te(nt * nt, 0.0), ts(nt * nt, 0.0);
        bool any_sig = false;
        for (size_t a = 0; a < eps_rows.size(); a++) {
            for (size_t b = 0; b < eps_rows[a].size(); b++) te[a * nt + b] = eps_rows[a][b];
            for (size_t b = 0; b < sig_rows[a].size(); b++) ts[a * nt + b] = sig_rows[a][b];
            any_sig = any_sig || !sig_rows[a].empty();
        }
        parm_host_check(parm_set_pair_table(h, (uint32_t)nt, te.data(), any_sig ? ts.data() : nullptr),
                        "parm_set_pair_table");
        rows_dirty = false;
        interaction_dirty = true;
    }
    if (interaction_dirty && nmembers > 0) {
        if (any_ldiam) parm_host_check(parm_set_list_diameters(h, ldiam.data()), "parm_set_list_diameters");
        // members without an NListed carry no parameters: any law with zero
        // epsilon gives them no force
        const int k = kind >= 0 ? kind : PARM_REPULSION;
        const size_t np = PARM_NPARAM(k), n = atomv->size();
        std::vector<double> packed(np * n);
        for (size_t i = 0; i < n; i++)
            for (size_t q = 0; q < np; q++) packed[np * i + q] = params[5 * i + q];
        parm_host_check(parm_set_interaction(h, k, packed.data(), rank.data(), skin_), "parm_set_interaction");
        interaction_dirty = false;
    }
    for (auto& pr : pending_ignores) parm_host_check(parm_nlist_ignore(h, pr.first, pr.second), "parm_nlist_ignore");
    pending_ignores.clear();
    parm_host_check(parm_set_atoms(h, atomv->records(), 4 * NDIM + 1, PARM_X | PARM_V | PARM_A | PARM_F | PARM_M),
                    "parm_set_atoms");
}

void GpuLink::pull() {
    parm_host_check(parm_get_atoms(h, atomv->records(), 4 * NDIM + 1, PARM_X | PARM_V | PARM_A | PARM_F | PARM_M),
                    "parm_get_atoms");
}

void GpuLink::sync_box() {
    std::vector<double> Lg(NDIM);
    parm_host_check(parm_get_boxes(h, Lg.data()), "parm_get_boxes");
    OriginBox& ob = *std::dynamic_pointer_cast<OriginBox>(bx);
    Vec v;
    for (int d = 0; d < NDIM; d++) v[d] = Lg[d];
    ob.resize_to(v);
    lastbox = Lg;
}

// ---------------------------------------------------------------------------
// NeighborList
NeighborList::NeighborList(sptr<Box> box, sptr<AtomVec> atoms, const flt skin)
    : link(new GpuLink(box, atoms, skin)) {}

bool NeighborList::update_list(bool force) {
    link->push();
    link->touch();
    uint8_t rebuilt = 0;
    parm_host_check(parm_nlist_update(link->handle(), force ? 1 : 0, &rebuilt), "parm_nlist_update");
    return rebuilt != 0;
}

uint NeighborList::which() {
    link->push();
    uint32_t w = 0;
    parm_host_check(parm_nlist_which(link->handle(), &w), "parm_nlist_which");
    return w;
}

uint NeighborList::numpairs() {
    link->push();
    uint64_t np = 0;
    parm_host_check(parm_nlist_numpairs(link->handle(), &np), "parm_nlist_numpairs");
    return (uint)np;
}

const std::vector<IDPair>& NeighborList::pairs() {
    if (cache_epoch == link->epoch()) return cache;
    link->push();
    uint64_t np = 0;
    parm_host_check(parm_nlist_pairs(link->handle(), 0, nullptr, 0, &np), "parm_nlist_pairs");
    std::vector<uint32_t> p(2 * np);
    parm_host_check(parm_nlist_pairs(link->handle(), 0, p.data(), np, &np), "parm_nlist_pairs");
    cache.clear();
    cache.reserve(np);
    AtomVec& av = *link->atoms();
    for (uint64_t k = 0; k < np; k++) cache.emplace_back(av.get_id(p[2 * k]), av.get_id(p[2 * k + 1]));
    cache_epoch = link->epoch();
    return cache;
}

// ---------------------------------------------------------------------------
// mean-square displacement (RsqTracker)
RsqTracker::RsqTracker(sptr<AtomGroup> atoms, std::vector<unsigned long> ns, bool usecom)
    : atoms(atoms), usecom(usecom) {
    if (ns.empty()) throw std::invalid_argument("RsqTracker: no time windows");
    for (unsigned long n : ns) skips.push_back((uint64_t)n);
    uint32_t n = atoms->size();
    parm_host_check(parm_create(&h, NDIM, 1, &n, PARM_FP64), "parm_create");
    // positions are measured unwrapped: the box is not used
    std::vector<double> L(NDIM, 1.0);
    parm_host_check(parm_set_boxes(h, L.data()), "parm_set_boxes");
    reset();
}

RsqTracker::~RsqTracker() {
    if (link) {
        parm_rsq_stop(link->handle());   // no throw from a destructor
        link->release_rsq(this);
    }
    if (h) parm_destroy(h);
}

void RsqTracker::push() {
    const uint n = atoms->size();
    const size_t stride = 4 * NDIM + 1;
    buf.assign((size_t)n * stride, 0.0);
    for (uint i = 0; i < n; i++) {
        const Atom& a = (*atoms)[i];
        for (int d = 0; d < NDIM; d++) buf[(size_t)i * stride + d] = a.x[d];
        buf[(size_t)i * stride + 4 * NDIM] = a.m;
    }
    parm_host_check(parm_set_atoms(h, buf.data(), stride, PARM_X | PARM_M), "parm_set_atoms");
}

void RsqTracker::reset() {
    if (link) {
        link->push();
    } else {
        push();
    }
    parm_host_check(parm_rsq_start(active(), skips.data(), (uint32_t)skips.size(), usecom ? 1 : 0),
                    "parm_rsq_start");
    const uint n = atoms->size();
    start.assign((size_t)n * NDIM, 0.0);
    for (uint i = 0; i < n; i++)
        for (int d = 0; d < NDIM; d++) start[(size_t)i * NDIM + d] = (*atoms)[i].x[d];
    nupdates = 0;
}

void RsqTracker::update(Box&) {
    if (link) {
        link->push();
    } else {
        push();
    }
    parm_host_check(parm_rsq_update(active()), "parm_rsq_update");
    nupdates++;
}

bool RsqTracker::bind(const sptr<GpuLink>& l) {
    if (link) return link == l;
    if (!l || static_cast<AtomGroup*>(l->atoms().get()) != atoms.get() || nupdates != 0) return false;
    const uint n = atoms->size();
    for (uint i = 0; i < n; i++)
        for (int d = 0; d < NDIM; d++)
            if (!((*atoms)[i].x[d] == start[(size_t)i * NDIM + d])) return false;
    if (!l->claim_rsq(this)) return false;
    l->push();
    if (parm_rsq_start(l->handle(), skips.data(), (uint32_t)skips.size(), usecom ? 1 : 0) != PARM_OK) {
        l->release_rsq(this);
        return false;
    }
    link = l;
    parm_destroy(h);
    h = nullptr;
    return true;
}

std::vector<double> RsqTracker::get(int what, size_t per_window) {
    std::vector<double> v(skips.size() * per_window);
    parm_host_check(parm_rsq_get(active(), what, v.data()), "parm_rsq_get");
    return v;
}

std::vector<VecRows> RsqTracker::rows(int what) {
    const size_t n = atoms->size();
    std::vector<double> v = get(what, n * NDIM);
    std::vector<VecRows> out;
    for (size_t j = 0; j < skips.size(); j++) {
        VecRows m(n);
        for (size_t i = 0; i < n; i++)
            for (int d = 0; d < NDIM; d++) m(i, d) = v[(j * n + i) * NDIM + d];
        out.push_back(m);
    }
    return out;
}

std::vector<std::vector<flt>> RsqTracker::lists(int what) {
    const size_t n = atoms->size();
    std::vector<double> v = get(what, n);
    std::vector<std::vector<flt>> out;
    for (size_t j = 0; j < skips.size(); j++) out.emplace_back(v.begin() + j * n, v.begin() + (j + 1) * n);
    return out;
}

std::vector<VecRows> RsqTracker::xyz2() { return rows(PARM_RSQ_XYZ2); }
std::vector<VecRows> RsqTracker::xyz4() { return rows(PARM_RSQ_XYZ4); }
std::vector<std::vector<flt>> RsqTracker::r2() { return lists(PARM_RSQ_R2); }
std::vector<std::vector<flt>> RsqTracker::r4() { return lists(PARM_RSQ_R4); }
std::vector<flt> RsqTracker::counts() { return get(PARM_RSQ_COUNTS, 1); }

// ---------------------------------------------------------------------------
// EnergyTracker (src/constraints.cpp:366-402)
void EnergyTracker::update(Box& box) {
    if (n_skipped + 1 < n_skip) {
        n_skipped += 1;
        return;
    }
    n_skipped = 0;
    const uint Natoms = atoms->size();
    flt curU = 0, curK = 0;
    for (uint i = 0; i < Natoms; ++i) {
        Atom& curatom = atoms->get(i);
        curK += curatom.v.squaredNorm() * curatom.m / 2;
    }
    for (auto& it : interactions) curU += it->energy(box);
    curU -= U0;
    Ks += curK;
    Us += curU;
    Es += curK + curU;
    Ksq += curK * curK;
    Usq += curU * curU;
    Esq += (curK + curU) * (curK + curU);
    N++;
}

void EnergyTracker::set_U0(Box& box) {
    flt curU = 0;
    for (auto& it : interactions) curU += it->energy(box);
    set_U0(curU);
}

// ---------------------------------------------------------------------------
// interaction quantities
flt gpu_evaluate(GpuLink& link, int what) {
    link.push();
    double v = 0.0;
    parm_host_check(parm_evaluate(link.handle(), what, &v), "parm_evaluate");
    return v;
}

Matrix gpu_stress(GpuLink& link) {
    link.push();
    double v[NDIM * NDIM];
    parm_host_check(parm_evaluate(link.handle(), PARM_EVAL_STRESS, v), "parm_evaluate");
    Matrix m;
    for (int a = 0; a < NDIM; a++)
        for (int b = 0; b < NDIM; b++) m(a, b) = v[a * NDIM + b];
    return m;
}

void gpu_add_forces(GpuLink& link) {
    AtomVec& av = *link.atoms();
    std::vector<Vec> f0(av.size());
    bool nonzero = false;
    for (uint i = 0; i < av.size(); i++) {
        f0[i] = av[i].f;
        nonzero |= f0[i] != Vec::Zero();
    }
    link.push();
    link.touch();
    parm_host_check(parm_set_forces(link.handle(), 0), "parm_set_forces");
    link.pull();
    if (nonzero)
        for (uint i = 0; i < av.size(); i++) av[i].f = f0[i] + av[i].f;
}

// ---------------------------------------------------------------------------
// Collection
Collection::Collection(sptr<Box> box, sptr<AtomVec> atoms, std::vector<sptr<Interaction>> is,
                       std::vector<sptr<StateTracker>> ts, std::vector<sptr<Constraint>> cs, bool should_initialize)
    : box(box), atoms(atoms), interactions(is), trackers(ts) {
    if (!cs.empty()) throw std::invalid_argument("parm_gb300: constraints are not supported on the GPU path");
    attach();
    if (should_initialize) initialize();
}

void Collection::attach() {
    sptr<GpuLink> found;
    for (auto& it : interactions) {
        GpuInteraction* gi = dynamic_cast<GpuInteraction*>(it.get());
        if (!gi)
            throw std::invalid_argument("parm_gb300: a Collection steps its atoms on the GPU; its interaction must be "
                                        "an NListed interaction");
        sptr<GpuLink> l = gi->gpu();
        if (found && l != found)
            throw std::invalid_argument("parm_gb300: one NListed interaction (one neighbour list) per Collection");
        found = l;
    }
    for (auto& t : trackers) {
        // other trackers are updated on the host after every step
        auto nl = std::dynamic_pointer_cast<NeighborList>(t);
        if (!nl) continue;
        if (found && nl->gpu() != found)
            throw std::invalid_argument("parm_gb300: the tracker must be the interaction's NeighborList");
        found = nl->gpu();
    }
    if (found && found->atoms() != atoms)
        throw std::invalid_argument("parm_gb300: the interaction was built on another AtomVec");
    link = found;
    // mean-square-displacement trackers of these atoms move onto the
    // Collection's handle: the time steps update them on the GPU
    if (link)
        for (auto& t : trackers)
            if (auto r = std::dynamic_pointer_cast<RsqTracker>(t)) r->bind(link);
}

GpuLink& Collection::gpu() {
    if (!link) throw std::logic_error("parm_gb300: the Collection has no NListed interaction");
    return *link;
}

void Collection::update_trackers() {
    for (auto& t : trackers) t->update(*box);
}

void Collection::initialize() {
    update_trackers();
    set_forces(true);
    update_trackers();
}

void Collection::set_forces(bool constraints_and_a) {
    if (!link || interactions.empty()) {
        // no interaction: zero forces, a = f/m (src/collection.cpp:159-179)
        atoms->reset_forces();
        if (constraints_and_a)
            for (uint i = 0; i < atoms->size(); i++) (*atoms)[i].a = Vec::Zero();
        return;
    }
    link->push();
    link->touch();
    parm_host_check(parm_set_forces(link->handle(), constraints_and_a ? 1 : 0), "parm_set_forces");
    link->pull();
}

flt Collection::set_forces_get_pressure(bool constraints_and_a) {
    set_forces(constraints_and_a);
    flt p = 0;
    for (auto& it : interactions) p += it->pressure(*box);
    return p;
}

void Collection::timesteps(uint n) {
    for (uint k = 0; k < n; k++) timestep();
}

flt Collection::potential_energy() {
    flt E = 0;
    for (auto& it : interactions) E += it->energy(*box);
    return E;
}

flt Collection::energy() { return potential_energy() + kinetic_energy(); }

flt Collection::degrees_of_freedom() {
    int ndof = 0;
    for (uint i = 0; i < atoms->size(); i++) {
        const Atom& a = (*atoms)[i];
        if (a.m <= 0 || std::isinf(a.m)) continue;
        ndof += NDIM;
    }
    return ndof;
}

flt Collection::temp(bool minuscomv) {
    Vec v = Vec::Zero();
    if (minuscomv) v = com_velocity();
    int ndof = (int)degrees_of_freedom();
    if (minuscomv) ndof -= NDIM;
    return atoms->kinetic_energy(v) * 2 / ndof;
}

flt Collection::pressure() {
    const flt V = box->V();
    flt E = 2.0 * kinetic_energy();
    for (auto& it : interactions) E += it->pressure(*box);
    return E / V / flt(NDIM);
}

void Collection::scale_velocities(flt scaleby) {
    for (uint i = 0; i < atoms->size(); i++) {
        Atom& a = (*atoms)[i];
        if (a.m <= 0 || std::isinf(a.m)) continue;
        a.v *= scaleby;
    }
}

void Collection::scale_velocities_to_temp(flt T, bool minuscomv) {
    const flt t = temp(minuscomv);
    scale_velocities(std::sqrt(T / t));
}

void Collection::scale_velocities_to_energy(flt E) {
    const flt E0 = energy();
    const flt k0 = kinetic_energy();
    const flt goalkinetic = k0 + (E - E0);
    scale_velocities(std::sqrt(goalkinetic / k0));
}

void Collection::add_interaction(sptr<Interaction> inter) {
    interactions.push_back(inter);
    attach();
    update_trackers();
}

void Collection::add_tracker(sptr<StateTracker> track) {
    trackers.push_back(track);
    attach();
    update_trackers();
}

bool Collection::has_step_trackers() const {
    for (auto& t : trackers)
        if (!std::dynamic_pointer_cast<NeighborList>(t)) return true;
    return false;
}

// the trackers that the GPU time steps on handle `g` update themselves: the
// neighbour list and the mean-square-displacement trackers bound to `g`
static bool updated_by_steps(const sptr<StateTracker>& t, const GpuLink& g) {
    if (std::dynamic_pointer_cast<NeighborList>(t)) return true;
    auto r = std::dynamic_pointer_cast<RsqTracker>(t);
    return r && r->bound_to(&g);
}

void Collection::run_steps(uint n, const std::function<void(uint)>& step) {
    if (!n) return;
    GpuLink& g = gpu();
    g.push();
    g.touch();
    bool host_trackers = false;
    for (auto& t : trackers) host_trackers = host_trackers || !updated_by_steps(t, g);
    if (!host_trackers) {
        step(n);
        g.pull();
        return;
    }
    // the other trackers see the positions at the end of every step
    for (uint k = 0; k < n; k++) {
        step(1);
        g.pull();
        for (auto& t : trackers)
            if (!updated_by_steps(t, g)) t->update(*box);
    }
}

void CollectionVerlet::timesteps(uint n) {
    run_steps(n, [this](uint k) { parm_host_check(parm_verlet(gpu().handle(), dt, k), "parm_verlet"); });
}

CollectionDamped::CollectionDamped(sptr<Box> box, sptr<AtomVec> atoms, const flt dt, const flt damping,
                                   std::vector<sptr<Interaction>> is, std::vector<sptr<StateTracker>> ts,
                                   std::vector<sptr<Constraint>> cs)
    : Collection(box, atoms, is, ts, cs, false), dt(dt), damping(damping) {
    initialize();
}

void CollectionDamped::timesteps(uint n) {
    run_steps(n, [this](uint k) {
        parm_host_check(parm_damped(gpu().handle(), dt, damping, k), "parm_damped");
    });
}

CollectionSol::CollectionSol(sptr<Box> box, sptr<AtomVec> atoms, const flt dt, const flt damping,
                             const flt desired_temperature, std::vector<sptr<Interaction>> is,
                             std::vector<sptr<StateTracker>> ts, std::vector<sptr<Constraint>> cs)
    : Collection(box, atoms, is, ts, cs, false), dt(dt), damping(damping), desT(desired_temperature) {
    if (dt <= 0) throw std::invalid_argument("Collection::CollectionSol: dt >= 0");
    key = ((unsigned long long)parm_random_engine()() << 32) | parm_random_engine()();
    initialize();
}

void CollectionSol::timesteps(uint n) {
    run_steps(n, [this](uint k) {
        parm_host_check(parm_sol(gpu().handle(), dt, damping, desT, key, k), "parm_sol");
    });
}

// ---------------------------------------------------------------------------
// CollectionNLCG / CollectionNLCGV (src/collection.cpp:494-1168)
CollectionNLCG::CollectionNLCG(sptr<OriginBox> box, sptr<AtomVec> atoms, const flt dt, const flt P0,
                               std::vector<sptr<Interaction>> is, std::vector<sptr<StateTracker>> ts,
                               std::vector<sptr<Constraint>> cs, const flt kappa, const flt kmax, const uint secmax,
                               const flt seceps)
    : Collection(box, atoms, is, ts, cs),
      dt(dt),
      seceps(seceps),
      secmax(secmax),
      kappa(kappa),
      alphamax(2.0),
      afrac(0),
      dxmax(100),
      stepmax(1e-3),
      kmax(kmax),
      P0(P0),
      Knew(0),
      k(0),
      vl(0),
      fl(0),
      al(0),
      alpha(0),
      beta(0),
      betaused(0),
      dxsum(0),
      alphavmax(0),
      maxdV(0),
      sec(0) {}

static sptr<OriginBox> origin_box(sptr<Box> b) {
    sptr<OriginBox> ob = std::dynamic_pointer_cast<OriginBox>(b);
    if (!ob) throw std::invalid_argument("parm_gb300: the GPU minimisers need a periodic OriginBox");
    return ob;
}

CollectionNLCGV::CollectionNLCGV(sptr<Box> box, sptr<AtomVec> atoms, const flt dt, std::vector<sptr<Interaction>> is,
                                 std::vector<sptr<StateTracker>> ts, std::vector<sptr<Constraint>> cs, const flt kmax,
                                 const uint secmax, const flt seceps)
    : CollectionNLCG(origin_box(box), atoms, dt, 0.0, is, ts, cs, 10.0, kmax, secmax, seceps) {
    boxed = false;
    alphamax = 0;
    afrac = 0;
    dxmax = 0;
    stepmax = 0;
}

void CollectionNLCG::gpu_params(double* p) const {
    const double v[PARM_NLCG_NPARAM] = {dt, P0, kappa, kmax, (double)secmax, seceps, alphamax, afrac,
                                        dxmax, stepmax, maxdV};
    for (int q = 0; q < PARM_NLCG_NPARAM; q++) p[q] = v[q];
}

GpuLink& CollectionNLCG::gpu_push() {
    GpuLink& g = gpu();
    g.push();
    g.touch();
    double p[PARM_NLCG_NPARAM];
    gpu_params(p);
    if (inited != g.handle()) {
        parm_host_check(parm_nlcg_init(g.handle(), boxed ? 1 : 0, p), "parm_nlcg_init");
        inited = g.handle();
    } else {
        parm_host_check(parm_nlcg_set_params(g.handle(), p), "parm_nlcg_set_params");
    }
    const double st[PARM_NLCG_NSTATE] = {Knew, k, vl, fl, al, alpha, beta, betaused, dxsum, alphavmax, (double)sec};
    parm_host_check(parm_nlcg_set_state(g.handle(), st), "parm_nlcg_set_state");
    return g;
}

void CollectionNLCG::gpu_pull(GpuLink& g) {
    double st[PARM_NLCG_NSTATE];
    parm_host_check(parm_nlcg_get_state(g.handle(), st), "parm_nlcg_get_state");
    Knew = st[PARM_NLCG_S_KNEW];
    k = st[PARM_NLCG_S_K];
    vl = st[PARM_NLCG_S_VL];
    fl = st[PARM_NLCG_S_FL];
    al = st[PARM_NLCG_S_AL];
    alpha = st[PARM_NLCG_S_ALPHA];
    beta = st[PARM_NLCG_S_BETA];
    betaused = st[PARM_NLCG_S_BETAUSED];
    dxsum = st[PARM_NLCG_S_DXSUM];
    alphavmax = st[PARM_NLCG_S_ALPHAVMAX];
    sec = (uint)st[PARM_NLCG_S_SEC];
    g.pull();
    if (boxed) g.sync_box();
}

flt CollectionNLCG::get_length_squared() {
    if (!boxed) return 1.0;
#ifdef VEC2D
    return box->V();
#else
    return std::pow(box->V(), 2.0 / 3.0);
#endif
}

// the four sums of src/collection.cpp:651-705 (boxed) and 910-975 (fixed box)
static flt mobile_sum(AtomVec& av, Vec Atom::*p, Vec Atom::*q) {
    flt r = 0;
    for (uint i = 0; i < av.size(); i++) {
        Atom& a = av[i];
        if (a.m <= 0 || std::isinf(a.m)) continue;
        r += (a.*p).dot(a.*q);
    }
    return r;
}
flt CollectionNLCG::fdota() {
    const flt r = mobile_sum(*atoms, &Atom::f, &Atom::a);
    return boxed ? r / get_length_squared() + fl * al : r;
}
flt CollectionNLCG::fdotf() {
    const flt r = mobile_sum(*atoms, &Atom::f, &Atom::f);
    return boxed ? r / get_length_squared() + fl * fl : r;
}
flt CollectionNLCG::fdotv() {
    const flt r = mobile_sum(*atoms, &Atom::f, &Atom::v);
    return boxed ? r / get_length_squared() + fl * vl : r;
}
flt CollectionNLCG::vdotv() {
    const flt r = mobile_sum(*atoms, &Atom::v, &Atom::v);
    return boxed ? r / get_length_squared() + vl * vl : r;
}

// CollectionNLCG::kinetic_energy (collection.cpp:572-587): masses ignored
flt CollectionNLCG::kinetic_energy() {
    flt E = 0;
    const flt Lfac = std::exp(vl / (kappa * NDIM));
    for (uint i = 0; i < atoms->size(); i++) {
        Atom& a = (*atoms)[i];
        if (a.m <= 0 || std::isinf(a.m)) continue;
        const Vec v = a.v + (a.x * Lfac);
        E += v.squaredNorm();
    }
    return E / 2.0;
}

// CollectionNLCG::pressure (collection.cpp:589-599), CollectionNLCGV::pressure (1007-1017)
flt CollectionNLCG::pressure() {
    const flt V = box->V();
    flt E = 0;
    for (auto& it : interactions) E += it->pressure(*box);
    return E / V / flt(NDIM);
}
flt CollectionNLCGV::pressure() { return CollectionNLCG::pressure(); }

flt CollectionNLCG::hamiltonian() { return potential_energy() + P0 * (box->V()); }

void CollectionNLCG::set_forces(bool constraints_and_a, bool setV) {
    if (!setV || !link || interactions.empty()) {
        // Collection::set_forces(false) and, when asked, the direction reset
        // of collection.cpp:553-564 on the Atom records
        Collection::set_forces(false);
        if (!constraints_and_a) return;
        for (uint i = 0; i < atoms->size(); i++) {
            Atom& a = (*atoms)[i];
            if (a.m <= 0 || std::isinf(a.m)) {
                a.v = Vec::Zero();
                a.a = Vec::Zero();
                continue;
            }
            a.a = a.f;
            a.v = a.f;
        }
        Knew = fdota();
        return;
    }
    GpuLink& g = gpu_push();
    parm_host_check(parm_nlcg_set_forces(g.handle(), constraints_and_a ? 1 : 0), "parm_nlcg_set_forces");
    gpu_pull(g);
}

void CollectionNLCG::reset() {
    GpuLink& g = gpu_push();
    parm_host_check(parm_nlcg_reset(g.handle()), "parm_nlcg_reset");
    gpu_pull(g);
}

void CollectionNLCG::descend() {
    GpuLink& g = gpu_push();
    parm_host_check(parm_nlcg_descend(g.handle()), "parm_nlcg_descend");
    gpu_pull(g);
    for (auto& t : trackers)
        if (!std::dynamic_pointer_cast<NeighborList>(t)) t->update(*box);
}

void CollectionNLCG::timesteps(uint n) {
    if (!n) return;
    GpuLink& g = gpu_push();
    if (!has_step_trackers()) {
        parm_host_check(parm_nlcg_timestep(g.handle(), n), "parm_nlcg_timestep");
        gpu_pull(g);
        return;
    }
    for (uint q = 0; q < n; q++) {
        parm_host_check(parm_nlcg_timestep(g.handle(), 1), "parm_nlcg_timestep");
        gpu_pull(g);
        for (auto& t : trackers)
            if (!std::dynamic_pointer_cast<NeighborList>(t)) t->update(*box);
    }
}
