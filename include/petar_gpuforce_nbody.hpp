// Header-only C++ wrapper of the device-resident tree step (pgf_nbody_* in
// petar_gpuforce.h).  Needs only the C header: unlike petar_gpuforce.hpp it
// does not depend on PeTar's record types.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "petar_gpuforce.h"

namespace petar_gpuforce {

// Device-resident tree step of singles (pgf_nbody_*): the particles stay in
// device memory; run() advances kick-drift-force-kick steps on the device,
// captured in one CUDA graph.  It stands for PeTar's host loop of kickOne
// (src/petar.hpp:1198-1212), driftSingle (src/petar.hpp:1326-1340) and
// treeSoftForce (src/petar.hpp:879-907) for singles without a hard part.
// Failures abort with the library's message, as the functors of
// petar_gpuforce.hpp do.
class DeviceTreeStep {
public:
    DeviceTreeStep(const pgf_nbody_config& cfg, int64_t n, const double* pos, const double* vel,
                   const double* mass, const double* r_search) {
        nbody_check(pgf_nbody_create(&cfg, n, pos, vel, mass, r_search, &h_), "pgf_nbody_create");
    }
    ~DeviceTreeStep() { pgf_nbody_destroy(h_); }
    DeviceTreeStep(const DeviceTreeStep&) = delete;
    DeviceTreeStep& operator=(const DeviceTreeStep&) = delete;

    // n_steps steps of size dt; returns the device milliseconds of the run.
    double run(int n_steps, double dt, bool graph = true) {
        double ms = 0.0;
        nbody_check(pgf_nbody_run(h_, n_steps, dt, graph ? 1 : 0, &ms), "pgf_nbody_run");
        return ms;
    }
    void force() { nbody_check(pgf_nbody_force(h_), "pgf_nbody_force"); }
    void get(double* pos, double* vel, double* acc, double* pot, int32_t* n_ngb) {
        nbody_check(pgf_nbody_get(h_, pos, vel, acc, pot, n_ngb), "pgf_nbody_get");
    }
    void set_state(const double* pos, const double* vel) {
        nbody_check(pgf_nbody_set_state(h_, pos, vel), "pgf_nbody_set_state");
    }
    void energy(double& kinetic, double& potential) {
        nbody_check(pgf_nbody_energy(h_, &kinetic, &potential), "pgf_nbody_energy");
    }
    pgf_nbody_stats stats() {
        pgf_nbody_stats s;
        nbody_check(pgf_nbody_get_stats(h_, &s), "pgf_nbody_get_stats");
        return s;
    }
    // Per-step sample: see pgf_nbody_set_sample / pgf_nbody_get_sample.
    void set_sample(int n_sample, const int64_t* particles, int max_records) {
        nbody_check(pgf_nbody_set_sample(h_, n_sample, particles, max_records), "pgf_nbody_set_sample");
    }
    int get_sample(pgf_nbody_sample* out) {
        int n = 0;
        nbody_check(pgf_nbody_get_sample(h_, &n, out), "pgf_nbody_get_sample");
        return n;
    }
    pgf_nbody* handle() { return h_; }

private:
    static void nbody_check(int code, const char* what) {
        if (code != PGF_OK) {
            std::fprintf(stderr, "petar_gpuforce: %s failed (%d): %s\n", what, code, pgf_nbody_last_error());
            std::abort();
        }
    }
    pgf_nbody* h_ = nullptr;
};

}  // namespace petar_gpuforce
