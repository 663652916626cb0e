// G4CXOpticks_gb.hh : header-only C++ host interface shaped like the reference's integration API, over the C ABI.
//
// A Geant4 application written against the reference keeps its call sequence:
//
//     gbo::G4CXOpticks* gx = gbo::G4CXOpticks::SetGeometry(desc);       // g4cx/G4CXOpticks.hh:49
//     gbo::SEvt::AddGenstep(q6);                                         // sysrap/SEvt.hh:487 (thread-safe)
//     gx->simulate(eventID, false);                                      // g4cx/G4CXOpticks.hh:95
//     int64_t n = gbo::SEvt::GetNumHit(0);                               // sysrap/SEvt.cc:2050
//     gbo_sphoton hit; gbo::SEvt::getHit(hit, i);                        // sysrap/SEvt.cc:4991
//     gx->reset(eventID);                                                // g4cx/G4CXOpticks.hh:96
//
// The only difference is SetGeometry's argument: the reference translates a G4VPhysicalVolume tree itself
// (g4cx/G4CXOpticks.cc:315-346); here the caller passes the CSGFoundry-layout arrays and optical tables that
// translation produces.  Failures throw std::runtime_error carrying the library's message (the reference asserts).
#pragma once

#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbo_gensteps.hh"
#include "gbopticks.h"

namespace gbo {

inline void check(int rc, const char* what)
{
    if (rc != GBO_OK) throw std::runtime_error(std::string(what) + ": " + gbo_last_error());
}

class SEvt {
public:
    static void AddGenstep(const gbo_quad6& q)
    {
        std::lock_guard<std::mutex> lock(mutex());
        gensteps().push_back(q);
    }
    static void SetInputPhoton(const gbo_sphoton* p, size_t n)
    {
        std::lock_guard<std::mutex> lock(mutex());
        input().assign(p, p + n);
        gensteps().clear();
        gbo_quad6 g = {};
        g.q[0].i[0] = GBO_GS_INPUT_PHOTON;
        g.q[0].u[3] = (uint32_t)n;
        gensteps().push_back(g);
    }
    // the gensteps collected for the next simulate (SEvt::GetNumGenstepFromGenstep / GetGenstep, in a copy)
    static int64_t GetNumGenstepFromGenstep(int /*eidx*/)
    {
        std::lock_guard<std::mutex> lock(mutex());
        return (int64_t)gensteps().size();
    }
    static std::vector<gbo_quad6> GetGenstep(int /*eidx*/)
    {
        std::lock_guard<std::mutex> lock(mutex());
        return gensteps();
    }
    static int64_t GetNumHit(int /*eidx*/)
    {
        gbo_engine* e = engine();
        return e ? gbo_num_hit(e) : 0;
    }
    static void getHit(gbo_sphoton& hit, unsigned idx)
    {
        std::vector<gbo_sphoton>& h = hits();
        if (h.empty() || idx >= h.size()) {
            const int64_t n = GetNumHit(0);
            h.resize((size_t)(n > 0 ? n : 0));
            if (n > 0) check(gbo_copy_hits(engine(), h.data(), 0, n), "gbo_copy_hits");
        }
        if (idx >= h.size()) throw std::out_of_range("SEvt::getHit index beyond the hits of this event");
        hit = h[idx];
    }
    static void Clear()
    {
        std::lock_guard<std::mutex> lock(mutex());
        gensteps().clear();
        input().clear();
        hits().clear();
    }

private:
    friend class G4CXOpticks;
    static std::mutex& mutex() { static std::mutex m; return m; }
    static std::vector<gbo_quad6>& gensteps() { static std::vector<gbo_quad6> v; return v; }
    static std::vector<gbo_sphoton>& input() { static std::vector<gbo_sphoton> v; return v; }
    static std::vector<gbo_sphoton>& hits() { static std::vector<gbo_sphoton> v; return v; }
    static gbo_engine*& engine() { static gbo_engine* e = nullptr; return e; }
};

class G4CXOpticks {
public:
    static G4CXOpticks* SetGeometry(const gbo_geometry_desc& desc, const gbo_config* cfg = nullptr, int device = 0)
    {
        G4CXOpticks*& inst = instance();
        delete inst;
        inst = new G4CXOpticks(desc, cfg, device);
        return inst;
    }
    static G4CXOpticks* Get() { return instance(); }
    static void Finalize()
    {
        delete instance();
        instance() = nullptr;
    }

    void simulate(int eventID, bool reset_ = false)
    {
        std::vector<gbo_quad6> gs;
        std::vector<gbo_sphoton> inp;
        {
            std::lock_guard<std::mutex> lock(SEvt::mutex());
            gs = SEvt::gensteps();
            inp = SEvt::input();
            SEvt::hits().clear();
        }
        check(gbo_simulate(engine_, eventID, gs.data(), (int64_t)gs.size(), inp.empty() ? nullptr : inp.data(),
                           (int64_t)inp.size()),
              "G4CXOpticks::simulate");
        if (reset_) reset(eventID);
    }

    void reset(int eventID)
    {
        SEvt::Clear();
        check(gbo_reset(engine_, eventID), "G4CXOpticks::reset");
    }

    gbo_engine* engine() const { return engine_; }

    ~G4CXOpticks()
    {
        if (SEvt::engine() == engine_) SEvt::engine() = nullptr;
        gbo_engine_destroy(engine_);
    }

private:
    G4CXOpticks(const gbo_geometry_desc& desc, const gbo_config* cfg, int device)
    {
        check(gbo_engine_create(&desc, cfg, device, &engine_), "G4CXOpticks::SetGeometry");
        SEvt::engine() = engine_;
    }
    static G4CXOpticks*& instance() { static G4CXOpticks* p = nullptr; return p; }
    gbo_engine* engine_ = nullptr;
};

// U4::CollectGenstep_* (u4/U4.cc:159-185, :278-311): make the genstep from the step's values and add it to the
// event, honouring the reference's environment switches: U4__CollectGenstep_<name>_DISABLE collects nothing,
// U4__CollectGenstep_<name>_ZEROPHO collects the genstep with zero photons.
struct U4 {
    static void CollectGenstep_DsG4Scintillation_r4695(const TrackInfo& t, const StepPoints& s, uint32_t matline,
                                                       int32_t numPhotons, int32_t scnt, double ScintillationTime)
    {
        if (std::getenv("U4__CollectGenstep_DsG4Scintillation_r4695_DISABLE")) return;
        if (std::getenv("U4__CollectGenstep_DsG4Scintillation_r4695_ZEROPHO")) numPhotons = 0;
        SEvt::AddGenstep(MakeGenstep_DsG4Scintillation_r4695(t, s, matline, numPhotons, scnt, ScintillationTime));
    }
    static void CollectGenstep_G4Cerenkov_modified(const TrackInfo& t, const StepPoints& s, uint32_t matline,
                                                   int32_t numPhotons, double betaInverse, double pmin_eV,
                                                   double pmax_eV, double maxCos, double maxSin2,
                                                   double meanNumberOfPhotons1, double meanNumberOfPhotons2)
    {
        if (std::getenv("U4__CollectGenstep_G4Cerenkov_modified_DISABLE")) return;
        if (std::getenv("U4__CollectGenstep_G4Cerenkov_modified_ZEROPHO")) numPhotons = 0;
        SEvt::AddGenstep(MakeGenstep_G4Cerenkov_modified(t, s, matline, numPhotons, betaInverse, pmin_eV, pmax_eV,
                                                         maxCos, maxSin2, meanNumberOfPhotons1, meanNumberOfPhotons2));
    }
};

}  // namespace gbo
