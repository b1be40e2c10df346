// parm_gb300 host API: time-step loops with the interface of the reference's
// src/collection.hpp (wackywendell/parm), run on the GPU.
//
// A Collection here drives one GPU handle: its interaction is the NListed
// interaction of one AtomVec and its neighbour list, whose update the GPU
// steps make themselves (constraints and other interactions are outside this
// library and rejected).  timestep() uploads the Atom records, runs one step
// of the reference's algorithm on the GPU and downloads the records, so code
// that reads or edits atoms[i] between steps behaves as with the reference;
// timesteps(n) runs n steps with one upload and one download, or, when the
// Collection holds trackers of the host (EnergyTracker, the caller's own, or
// an RsqTracker it could not bind), one step at a time with the trackers
// updated after each, as the reference's timestep does.  An RsqTracker of
// the Collection's own AtomVec is bound to its handle when the Collection is
// made (RsqTracker::bind) and updated inside the GPU steps.
#ifndef PARM_GB300_COLLECTION_HPP
#define PARM_GB300_COLLECTION_HPP

#include <functional>
#include <vector>

#include "constraints.hpp"

//! Constraints are not part of this library; the type exists so that
//! constructor signatures match the reference's.
class Constraint {
   public:
    virtual ~Constraint() {}
};

//! Base of the time-step loops (src/collection.hpp:23-131, src/collection.cpp:1-180).
class Collection {
   protected:
    sptr<Box> box;
    sptr<AtomVec> atoms;
    std::vector<sptr<Interaction>> interactions;
    std::vector<sptr<StateTracker>> trackers;
    sptr<GpuLink> link;
    void attach();
    GpuLink& gpu();
    //! trackers besides the neighbour list (updated after every step)
    bool has_step_trackers() const;
    //! push, step(k) for n steps (one at a time when such trackers exist), pull
    void run_steps(uint n, const std::function<void(uint)>& step);

   public:
    Collection(sptr<Box> box, sptr<AtomVec> atoms,
               std::vector<sptr<Interaction>> is = std::vector<sptr<Interaction>>(),
               std::vector<sptr<StateTracker>> ts = std::vector<sptr<StateTracker>>(),
               std::vector<sptr<Constraint>> cs = std::vector<sptr<Constraint>>(),
               bool should_initialize = true);
    virtual ~Collection() {}

    //! update_trackers(); set_forces(true); update_trackers() (src/collection.cpp:13-19)
    void initialize();
    void update_trackers();
    virtual void set_forces(bool constraints_and_a = true);
    virtual flt set_forces_get_pressure(bool constraints_and_a = true);
    virtual void timestep() = 0;
    //! n time steps with one upload and one download of the Atom records
    virtual void timesteps(uint n);

    flt potential_energy();
    flt energy();
    virtual flt kinetic_energy() { return atoms->kinetic_energy(); }
    flt degrees_of_freedom();
    virtual flt temp(bool minuscomv = true);
    virtual flt pressure();
    Vec com_velocity() { return atoms->com_velocity(); }
    void reset_com_velocity() { atoms->reset_com_velocity(); }
    void scale_velocities(flt scaleby);
    void scale_velocities_to_temp(flt T, bool minuscomv = true);
    void scale_velocities_to_energy(flt E);

    virtual void add_interaction(sptr<Interaction> inter);
    virtual void add_tracker(sptr<StateTracker> track);
};

//! Velocity Verlet (src/collection.hpp:360-374, src/collection.cpp:442-469).
class CollectionVerlet : public Collection {
   protected:
    flt dt;

   public:
    CollectionVerlet(sptr<Box> box, sptr<AtomVec> atoms, const flt dt,
                     std::vector<sptr<Interaction>> is = std::vector<sptr<Interaction>>(),
                     std::vector<sptr<StateTracker>> ts = std::vector<sptr<StateTracker>>(),
                     std::vector<sptr<Constraint>> cs = std::vector<sptr<Constraint>>())
        : Collection(box, atoms, is, ts, cs), dt(dt) {}
    void timestep() override { timesteps(1); }
    void timesteps(uint n) override;
    void set_dt(flt newdt) { dt = newdt; }
};

//! Damped velocity Verlet (src/collection.hpp:273-326, src/collection.cpp:324-381).
class CollectionDamped : public Collection {
   protected:
    flt dt, damping;

   public:
    CollectionDamped(sptr<Box> box, sptr<AtomVec> atoms, const flt dt, const flt damping,
                     std::vector<sptr<Interaction>> is = std::vector<sptr<Interaction>>(),
                     std::vector<sptr<StateTracker>> ts = std::vector<sptr<StateTracker>>(),
                     std::vector<sptr<Constraint>> cs = std::vector<sptr<Constraint>>());
    void timestep() override { timesteps(1); }
    void timesteps(uint n) override;
};

//! Langevin dynamics (src/collection.hpp:205-271, src/collection.cpp:230-322).
//! The noise comes from a counter-based generator (one stream per handle,
//! keyed from the seeded host engine), not from the reference's Boost stream.
class CollectionSol : public Collection {
   protected:
    flt dt, damping, desT;
    unsigned long long key;

   public:
    CollectionSol(sptr<Box> box, sptr<AtomVec> atoms, const flt dt, const flt damping,
                  const flt desired_temperature,
                  std::vector<sptr<Interaction>> is = std::vector<sptr<Interaction>>(),
                  std::vector<sptr<StateTracker>> ts = std::vector<sptr<StateTracker>>(),
                  std::vector<sptr<Constraint>> cs = std::vector<sptr<Constraint>>());
    void timestep() override { timesteps(1); }
    void timesteps(uint n) override;
    void set_damping(flt d) { damping = d; }
    void set_temperature(flt T) { desT = T; }
};

//! Conjugate-gradient energy minimisation of positions and the box's
//! log-volume, H = U + P0 V (src/collection.hpp:400-475,
//! src/collection.cpp:494-829), run on the GPU (parm_nlcg_*): each time step
//! (the secant line search included) is one GPU call.  The public members
//! are the reference's; they are sent to the GPU before and read back after
//! every call, so code that reads or sets them behaves as with the
//! reference.  The box (an OriginBox) is rescaled on the GPU and copied back.
//! Trackers other than the neighbour list are updated after each time step.
class CollectionNLCG : public Collection {
   public:
    flt dt;
    flt seceps;
    uint secmax;
    flt kappa;
    flt alphamax, afrac, dxmax, stepmax, kmax;
    flt P0;
    flt Knew;
    flt k;
    flt vl, fl, al;
    flt alpha, beta, betaused, dxsum, alphavmax, maxdV;
    uint sec;

    CollectionNLCG(sptr<OriginBox> box, sptr<AtomVec> atoms, const flt dt, const flt P0,
                   std::vector<sptr<Interaction>> is = std::vector<sptr<Interaction>>(),
                   std::vector<sptr<StateTracker>> ts = std::vector<sptr<StateTracker>>(),
                   std::vector<sptr<Constraint>> cs = std::vector<sptr<Constraint>>(), const flt kappa = 10.0,
                   const flt kmax = 1000, const uint secmax = 40, const flt seceps = 1e-20);

    //! host sums over the Atom records, as the reference defines them
    flt get_length_squared();
    flt fdota();
    flt fdotf();
    flt fdotv();
    flt vdotv();
    flt kinetic_energy() override;   // masses ignored
    flt pressure() override;
    flt hamiltonian();
    void set_forces(bool constraints_and_a = true) override { set_forces(constraints_and_a, true); }
    void set_forces(bool constraints_and_a, bool setV);

    void timestep() override { timesteps(1); }
    void timesteps(uint n) override;
    void descend();
    void reset();

    void set_dt(flt newdt) {
        dt = newdt;
        reset();
    }
    void set_pressure_goal(flt P) {
        P0 = P;
        reset();
    }
    flt get_pressure_goal() { return P0; }
    void set_kappa(flt kk) {
        kappa = kk;
        reset();
    }
    void set_max_alpha(flt a) { alphamax = a; }
    void set_max_alpha_fraction(flt a) { afrac = a; }
    void set_max_dx(flt d) { dxmax = d; }
    void set_max_step(flt m) { stepmax = m; }

   protected:
    bool boxed = true;
    parm_system* inited = nullptr;   // the handle the GPU minimiser was set up on
    //! push the Atom records, the box and this object's members to the GPU
    GpuLink& gpu_push();
    //! read members, Atom records and the box back
    void gpu_pull(GpuLink& g);
    void gpu_params(double* p) const;
};

//! Conjugate-gradient energy minimisation of positions in a fixed box
//! (src/collection.hpp:490-566, src/collection.cpp:877-1168), on the GPU.
class CollectionNLCGV : public CollectionNLCG {
   public:
    CollectionNLCGV(sptr<Box> box, sptr<AtomVec> atoms, const flt dt,
                    std::vector<sptr<Interaction>> is = std::vector<sptr<Interaction>>(),
                    std::vector<sptr<StateTracker>> ts = std::vector<sptr<StateTracker>>(),
                    std::vector<sptr<Constraint>> cs = std::vector<sptr<Constraint>>(), const flt kmax = 1000,
                    const uint secmax = 10, const flt seceps = 1e-4);
    flt kinetic_energy() override { return atoms->kinetic_energy(); }
    flt pressure() override;
    void set_forces(bool constraints_and_a = true) override { Collection::set_forces(constraints_and_a); }
    void set_dt(flt newdt) {
        dt = newdt;
        reset();
    }
};

#endif
