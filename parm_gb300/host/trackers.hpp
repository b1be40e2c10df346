// parm_gb300 host API: the neighbour list with the interface of the
// reference's src/trackers.hpp (wackywendell/parm), backed by the GPU.
//
// One GPU handle (parm_system, include/parm_gb300.h) serves one AtomVec and
// the one NListed interaction and NeighborList built on it.  `GpuLink` holds
// that handle and the host-side description of the interaction, and moves
// the Atom records between host and GPU around every GPU operation.
#ifndef PARM_GB300_TRACKERS_HPP
#define PARM_GB300_TRACKERS_HPP

#include <set>
#include <utility>
#include <vector>

#include "box.hpp"
#include "parm_gb300.h"

//! Precision of GPU handles created from now on: PARM_FP64 (default, the
//! reference's results) or PARM_MIXED.  The environment variable
//! PARM_PRECISION=mixed sets the default.
void parm_host_set_precision(int precision);
int parm_host_precision();

//! Throws std::runtime_error with parm_last_error() when rc != PARM_OK.
void parm_host_check(int rc, const char* what);

class GpuLink {
   public:
    GpuLink(sptr<Box> box, sptr<AtomVec> atoms, flt skin);
    ~GpuLink();
    GpuLink(const GpuLink&) = delete;
    GpuLink& operator=(const GpuLink&) = delete;

    //! NListed::add: per-atom parameters (kind: PARM_LJCUT, ...; the first
    //! PARM_NPARAM(kind) of p) and the atom's position in the neighbour list
    //! (insertion order); `owner` is the NListed adding it (one NListed per
    //! neighbour list)
    void add(uint atom, int kind, const double p[5], const void* owner);
    //! the pair tables of the indexed kinds: the epsilons (and sigmas, or
    //! NULL) of the atoms of type `type`; atoms of one type must share them
    void set_type_row(uint type, const std::vector<flt>& eps, const std::vector<flt>* sig);
    //! NeighborList::add(atom, diameter): a list member with its own list
    //! diameter and no pair parameters (its pairs carry no force)
    void add_member(uint atom, double diameter);
    void ignore(uint a, uint b);
    uint ignored() const { return nignored; }
    //! upload box, interaction and Atom records (create the handle if needed)
    void push();
    //! download the Atom records
    void pull();
    //! copy the GPU's box (rescaled by a minimiser) into the host OriginBox
    void sync_box();
    parm_system* handle() { return h; }
    sptr<Box> box() { return bx; }
    sptr<AtomVec> atoms() { return atomv; }
    uint members() const { return nmembers; }
    flt skin() const { return skin_; }
    //! advanced by every operation that may change the pair list
    unsigned long long epoch() const { return epoch_; }
    void touch() { epoch_++; }
    //! the device tracker of this handle (parm_rsq_*) belongs to one RsqTracker
    bool claim_rsq(const void* who) {
        if (rsq_owner && rsq_owner != who) return false;
        rsq_owner = who;
        return true;
    }
    void release_rsq(const void* who) {
        if (rsq_owner == who) rsq_owner = nullptr;
    }

   private:
    sptr<Box> bx;
    sptr<AtomVec> atomv;
    flt skin_;
    parm_system* h = nullptr;
    int kind = -1;
    std::vector<double> params;   // five per atom
    std::vector<std::vector<double>> eps_rows, sig_rows;   // by type index (indexed kinds)
    double lastgamma = std::nan("");                       // shear sent to the GPU (LeesEdwardsBox)
    bool rows_dirty = false;
    std::vector<uint32_t> rank;
    std::vector<double> ldiam;   // explicit list diameters (NaN: the parameters' max_size())
    bool any_ldiam = false;
    const void* owner_ = nullptr;
    uint nmembers = 0;
    uint nignored = 0;
    bool interaction_dirty = false;
    std::vector<std::pair<uint, uint>> pending_ignores;
    std::vector<double> lastbox;
    unsigned long long epoch_ = 0;
    const void* rsq_owner = nullptr;
};

//! Something to update before or after each time step (src/trackers.hpp:9-16).
class StateTracker {
   public:
    virtual void update(Box& box) = 0;
    virtual ~StateTracker() {}
};

//! A pair of atoms of the neighbour list.
class IDPair {
   protected:
    AtomID a1, a2;

   public:
    IDPair() {}
    IDPair(AtomID a, AtomID b) : a1(a), a2(b) {}
    AtomID first() const { return a1; }
    AtomID last() const { return a2; }
};

//! Verlet neighbour list with displacement-triggered rebuild
//! (src/trackers.hpp:133-215, src/trackers.cpp:19-85).
class NeighborList : public StateTracker {
   public:
    NeighborList(sptr<Box> box, sptr<AtomVec> atoms, const flt skin);
    explicit NeighborList(sptr<GpuLink> link) : link(link) {}
    void update(Box& newbox) override { update_list(false); }
    //! rebuild if forced or if the two largest displacements sum to >= skin;
    //! returns whether a rebuild happened
    bool update_list(bool force = true);
    uint which();
    uint numpairs();
    void ignore(AtomID a, AtomID b) { link->ignore(a.n(), b.n()); }
    //! NeighborList::add(a, diameter) (src/trackers.hpp:194-201): a member
    //! with the given list diameter (NListed::add calls it with max_size())
    void add(AtomID a, flt diameter) { link->add_member(a.n(), diameter); }
    uint ignore_size() const { return link->ignored(); }
    uint size() const { return link->members(); }
    flt skin() const { return link->skin(); }
    AtomVec& vec() { return *link->atoms(); }
    //! the current pairs in the reference's order
    const std::vector<IDPair>& pairs();
    IDPair get(uint i) { return pairs().at(i); }
    std::vector<IDPair>::iterator begin() {
        pairs();
        return cache.begin();
    }
    std::vector<IDPair>::iterator end() {
        pairs();
        return cache.end();
    }
    sptr<GpuLink> gpu() { return link; }

   private:
    sptr<GpuLink> link;
    std::vector<IDPair> cache;
    unsigned long long cache_epoch = ~0ull;
};

//! Mean-square displacement over windows of ns[j] updates
//! (src/constraints.hpp:318-361, src/constraints.cpp:404-564), on the GPU
//! (parm_rsq_*): the tracker holds its own GPU handle and sends it the
//! atoms' positions and masses at each update.  A Collection updates it at
//! the end of every time step, as the reference's update_trackers does; a
//! Collection that steps the same AtomVec moves the tracker onto its own
//! handle (bind), where the time-step graphs update it with no copies and
//! several steps run in one call.
class RsqTracker : public StateTracker {
   public:
    RsqTracker(sptr<AtomGroup> atoms, std::vector<unsigned long> ns, bool usecom = true);
    ~RsqTracker() override;
    RsqTracker(const RsqTracker&) = delete;
    RsqTracker& operator=(const RsqTracker&) = delete;
    //! restart every window at the current positions
    void reset();
    void update(Box& box) override;
    //! Move the tracker onto the handle of a Collection that steps these
    //! same atoms on the GPU: the time steps then update it inside their
    //! graphs, with no records copied.  Done only while the tracker has not
    //! been updated since its last reset and the atoms have not moved since
    //! (nothing is lost); false otherwise, and the tracker stays on its own
    //! handle.
    bool bind(const sptr<GpuLink>& link);
    bool bound() const { return (bool)link; }
    bool bound_to(const GpuLink* l) const { return link.get() == l; }
    std::vector<VecRows> xyz2();
    std::vector<std::vector<flt>> r2();
    std::vector<VecRows> xyz4();
    std::vector<std::vector<flt>> r4();
    std::vector<flt> counts();

   private:
    sptr<AtomGroup> atoms;
    std::vector<uint64_t> skips;
    bool usecom;
    parm_system* h = nullptr;
    sptr<GpuLink> link;          // the Collection's handle, once bound
    std::vector<double> buf;
    std::vector<double> start;   // positions at the last reset
    unsigned long nupdates = 0;  // updates since the last reset
    parm_system* active() { return link ? link->handle() : h; }
    void push();
    std::vector<double> get(int what, size_t per_window);
    std::vector<VecRows> rows(int what);
    std::vector<std::vector<flt>> lists(int what);
};

#endif
