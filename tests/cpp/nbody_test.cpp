// Drives petar_gpuforce::DeviceTreeStep from C++: reads particles and a
// configuration, runs n_steps leapfrog steps in one CUDA graph, writes the
// final positions, accelerations, potentials and neighbour counts.
//
// Input (binary): int64 n, int64 n_steps, double dt, eps2, r_out, G, theta,
// int32 n_leaf_limit, n_group_limit, then pos[3n], vel[3n], mass[n],
// r_search[n].  Output: pos[3n], acc[3n], pot[n] (doubles), n_ngb[n] (int32).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "petar_gpuforce_nbody.hpp"

namespace {
template <class T>
void rd(std::FILE* f, T* p, size_t n) {
    if (std::fread(p, sizeof(T), n, f) != n) {
        std::fprintf(stderr, "short input\n");
        std::exit(2);
    }
}
}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: nbody_test in.bin out.bin\n");
        return 2;
    }
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t hdr[2];
    double par[5];
    int32_t lim[2];
    rd(f, hdr, 2);
    rd(f, par, 5);
    rd(f, lim, 2);
    const int64_t n = hdr[0];
    std::vector<double> pos(3 * n), vel(3 * n), mass(n), rs(n);
    rd(f, pos.data(), pos.size());
    rd(f, vel.data(), vel.size());
    rd(f, mass.data(), mass.size());
    rd(f, rs.data(), rs.size());
    std::fclose(f);

    pgf_nbody_config cfg{};
    cfg.eps2 = par[1];
    cfg.r_out = par[2];
    cfg.G = par[3];
    cfg.theta = par[4];
    cfg.n_leaf_limit = lim[0];
    cfg.n_group_limit = lim[1];
    cfg.precision = PGF_PRECISION_MIXED;
    cfg.kernel_variant = -1;
    cfg.list_capacity_factor = 2.0;
    petar_gpuforce::DeviceTreeStep step(cfg, n, pos.data(), vel.data(), mass.data(), rs.data());
    const int64_t probe[2] = {0, n - 1};
    step.set_sample(2, probe, (int)hdr[1] + 1);
    step.run((int)hdr[1], par[0], true);
    std::vector<pgf_nbody_sample> rec(2 * (hdr[1] + 1));
    const int n_rec = step.get_sample(rec.data());
    if (n_rec != (int)hdr[1]) {
        std::fprintf(stderr, "expected %lld sample records, got %d\n", (long long)hdr[1], n_rec);
        return 3;
    }
    for (int r = 0; r < 2 * n_rec; ++r)
        if (rec[r].n_ngb != rec[r].n_ngb64) {
            std::fprintf(stderr, "sample %d: neighbour counts differ\n", r);
            return 3;
        }
    std::vector<double> acc(3 * n), pot(n);
    std::vector<int32_t> nnb(n);
    step.get(pos.data(), nullptr, acc.data(), pot.data(), nnb.data());
    std::FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    std::fwrite(pos.data(), sizeof(double), pos.size(), o);
    std::fwrite(acc.data(), sizeof(double), acc.size(), o);
    std::fwrite(pot.data(), sizeof(double), pot.size(), o);
    std::fwrite(nnb.data(), sizeof(int32_t), nnb.size(), o);
    std::fclose(o);
    const pgf_nbody_stats s = step.stats();
    std::printf("steps %lld groups %lld cells %lld\n", (long long)s.steps, (long long)s.n_groups,
                (long long)s.n_cells);
    return 0;
}
