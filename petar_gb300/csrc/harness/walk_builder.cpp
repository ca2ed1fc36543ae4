// Interaction-list builder: the caller side of the soft-force kernels.
//
// PeTar gets its interaction lists from FDPS's long-range tree with symmetric
// r_search opening (PS::TreeForForceLong<...>::QuadrupoleWithSymmetrySearch,
// src/petar.hpp:619-623), walked group by group by
// calcForceAllAndWriteBackMultiWalkIndex (src/petar.hpp:894-899).  FDPS is not
// part of the reference tree, so this file restates what that caller hands to
// the dispatch functor:
//   * particles sorted along a Morton curve inside a cubic root cell,
//   * an octree whose cells split while they hold more than n_leaf_limit
//     particles,
//   * quadrupole moments per cell: mass, centre of mass and the raw second
//     moment sum m (x - c)(x - c)^T about the centre of mass (the convention
//     the quadrupole formulas in src/soft_force.hpp:160-200 assume), built
//     bottom-up from the children's moments as FDPS's moment pass does,
//   * i-groups: the first cells (top-down) holding at most n_group_limit
//     particles,
//   * per group, a walk that opens a cell when the squared distance from the
//     group's particle box to the cell's centre of mass is at most
//     (cell side / theta)^2, or when the r_search-expanded box of either side
//     overlaps the particle box of the other (symmetric search).  Opened leaves
//     contribute their particles as EPJ, unopened cells their moments as SPJ.
// The symmetric test uses the full r_search (not FDPS's 0.99 factor,
// src/ptcl.hpp:8) so that every pair with |xi-xj| < max(rs_i, rs_j) is an EPJ
// of the walk and list-based neighbour counts equal global counts.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

constexpr int kMaxLevel = 21;  // 3 x 21 bits of Morton key

struct Cell {
    int64_t begin, end;  // particle range in sorted order
    int level;
    int n_child;
    int child[8];
    double side;
    double mass;
    double mx[3];    // mass moment sum m x
    double com[3];
    double quad[6];  // xx, yy, zz, xy, xz, yz
    double in_lo[3], in_hi[3];
    double out_lo[3], out_hi[3];
    bool leaf;
};

inline uint64_t spread3(uint64_t v) {
    v &= 0x1fffff;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

struct WalkSet {
    int64_t n = 0;
    std::vector<int64_t> order;  // sorted position -> input index
    std::vector<Cell> cells;
    std::vector<int64_t> group_cell;
    std::vector<int64_t> group_begin;  // n_group + 1, sorted-order i ranges
    std::vector<int64_t> epj_disp;     // n_group + 1
    std::vector<int64_t> spj_disp;     // n_group + 1
    std::vector<int32_t> id_epj;
    std::vector<int32_t> id_spj;
};

inline double box_dist2_point(const double lo[3], const double hi[3], const double p[3]) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        double dd = 0.0;
        if (p[d] < lo[d]) dd = lo[d] - p[d];
        else if (p[d] > hi[d]) dd = p[d] - hi[d];
        s += dd * dd;
    }
    return s;
}

inline bool box_overlap(const double alo[3], const double ahi[3], const double blo[3], const double bhi[3]) {
    for (int d = 0; d < 3; ++d)
        if (alo[d] > bhi[d] || blo[d] > ahi[d]) return false;
    return true;
}

void build(WalkSet& ws, const double* pos, const double* mass, const double* rs, int64_t n,
           double theta, int n_leaf, int n_group) {
    ws.n = n;
    // Root cube.
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], pos[3 * i + d]);
            hi[d] = std::max(hi[d], pos[3 * i + d]);
        }
    double half = 0.0, cen[3];
    for (int d = 0; d < 3; ++d) {
        cen[d] = 0.5 * (lo[d] + hi[d]);
        half = std::max(half, 0.5 * (hi[d] - lo[d]));
    }
    half = half * 1.0001 + 1e-12;
    const double root_lo[3] = {cen[0] - half, cen[1] - half, cen[2] - half};
    const double scale = double(1 << kMaxLevel) / (2.0 * half);

    std::vector<std::pair<uint64_t, int64_t>> keys(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t k = 0;
        for (int d = 0; d < 3; ++d) {
            double f = (pos[3 * i + d] - root_lo[d]) * scale;
            int64_t c = (int64_t)f;
            if (c < 0) c = 0;
            if (c > (1 << kMaxLevel) - 1) c = (1 << kMaxLevel) - 1;
            k |= spread3((uint64_t)c) << (2 - d);
        }
        keys[i] = {k, i};
    }
    std::sort(keys.begin(), keys.end());
    ws.order.resize(n);
    std::vector<uint64_t> skey(n);
    for (int64_t i = 0; i < n; ++i) {
        ws.order[i] = keys[i].second;
        skey[i] = keys[i].first;
    }
    keys.clear();
    keys.shrink_to_fit();

    // Sorted copies for the moment and box passes.
    std::vector<double> sp(3 * n), sm(n), sr(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t o = ws.order[i];
        for (int d = 0; d < 3; ++d) sp[3 * i + d] = pos[3 * o + d];
        sm[i] = mass[o];
        sr[i] = rs[o];
    }

    // Top-down octree, breadth first.
    ws.cells.clear();
    Cell root{};
    root.begin = 0;
    root.end = n;
    root.level = 0;
    root.side = 2.0 * half;
    ws.cells.push_back(root);
    for (size_t c = 0; c < ws.cells.size(); ++c) {
        Cell cc = ws.cells[c];
        int64_t cnt = cc.end - cc.begin;
        cc.n_child = 0;
        cc.leaf = (cnt <= n_leaf) || (cc.level >= kMaxLevel);
        if (!cc.leaf) {
            int shift = 3 * (kMaxLevel - 1 - cc.level);
            int64_t b = cc.begin;
            for (int oct = 0; oct < 8; ++oct) {
                int64_t e = b;
                while (e < cc.end && (int)((skey[e] >> shift) & 7) == oct) ++e;
                if (e > b) {
                    Cell ch{};
                    ch.begin = b;
                    ch.end = e;
                    ch.level = cc.level + 1;
                    ch.side = cc.side * 0.5;
                    cc.child[cc.n_child++] = (int)ws.cells.size();
                    ws.cells.push_back(ch);
                }
                b = e;
            }
        }
        ws.cells[c] = cc;
    }

    // Moments and boxes, bottom-up.  A leaf sums its particles in sorted
    // order; a parent combines its children in child order: mass and the mass
    // moment m x are added, the centre of mass is their quotient, and the
    // second moment about it follows from the children's by the parallel-axis
    // term m_c (c_c - c)(c_c - c)^T.  Built without FMA contraction, so the
    // device builder reproduces every bit of it.
    const int64_t nc = (int64_t)ws.cells.size();
    for (int64_t c = nc - 1; c >= 0; --c) {
        Cell& cc = ws.cells[c];
        double m = 0, mx[3] = {0, 0, 0}, q[6] = {0, 0, 0, 0, 0, 0};
        for (int d = 0; d < 3; ++d) {
            cc.in_lo[d] = cc.out_lo[d] = 1e300;
            cc.in_hi[d] = cc.out_hi[d] = -1e300;
        }
        if (cc.leaf) {
            for (int64_t i = cc.begin; i < cc.end; ++i) {
                m += sm[i];
                for (int d = 0; d < 3; ++d) {
                    const double x = sp[3 * i + d];
                    mx[d] += sm[i] * x;
                    cc.in_lo[d] = std::min(cc.in_lo[d], x);
                    cc.in_hi[d] = std::max(cc.in_hi[d], x);
                    cc.out_lo[d] = std::min(cc.out_lo[d], x - sr[i]);
                    cc.out_hi[d] = std::max(cc.out_hi[d], x + sr[i]);
                }
            }
        } else {
            for (int k = 0; k < cc.n_child; ++k) {
                const Cell& ch = ws.cells[cc.child[k]];
                m += ch.mass;
                for (int d = 0; d < 3; ++d) {
                    mx[d] += ch.mx[d];
                    cc.in_lo[d] = std::min(cc.in_lo[d], ch.in_lo[d]);
                    cc.in_hi[d] = std::max(cc.in_hi[d], ch.in_hi[d]);
                    cc.out_lo[d] = std::min(cc.out_lo[d], ch.out_lo[d]);
                    cc.out_hi[d] = std::max(cc.out_hi[d], ch.out_hi[d]);
                }
            }
        }
        cc.mass = m;
        for (int d = 0; d < 3; ++d) {
            cc.mx[d] = mx[d];
            if (m > 0) cc.com[d] = mx[d] / m;
            else cc.com[d] = 0.5 * (cc.in_lo[d] + cc.in_hi[d]);
        }
        if (cc.leaf) {
            for (int64_t i = cc.begin; i < cc.end; ++i) {
                const double dx = sp[3 * i] - cc.com[0], dy = sp[3 * i + 1] - cc.com[1],
                             dz = sp[3 * i + 2] - cc.com[2];
                q[0] += sm[i] * dx * dx;
                q[1] += sm[i] * dy * dy;
                q[2] += sm[i] * dz * dz;
                q[3] += sm[i] * dx * dy;
                q[4] += sm[i] * dx * dz;
                q[5] += sm[i] * dy * dz;
            }
        } else {
            for (int k = 0; k < cc.n_child; ++k) {
                const Cell& ch = ws.cells[cc.child[k]];
                const double dx = ch.com[0] - cc.com[0], dy = ch.com[1] - cc.com[1], dz = ch.com[2] - cc.com[2];
                q[0] += ch.quad[0] + ch.mass * dx * dx;
                q[1] += ch.quad[1] + ch.mass * dy * dy;
                q[2] += ch.quad[2] + ch.mass * dz * dz;
                q[3] += ch.quad[3] + ch.mass * dx * dy;
                q[4] += ch.quad[4] + ch.mass * dx * dz;
                q[5] += ch.quad[5] + ch.mass * dy * dz;
            }
        }
        for (int k = 0; k < 6; ++k) cc.quad[k] = q[k];
    }

    // i-groups in Morton order.
    ws.group_cell.clear();
    {
        std::vector<int64_t> stack{0};
        while (!stack.empty()) {
            int64_t c = stack.back();
            stack.pop_back();
            const Cell& cc = ws.cells[c];
            if (cc.end - cc.begin <= n_group || cc.leaf) {
                ws.group_cell.push_back(c);
            } else {
                for (int k = cc.n_child - 1; k >= 0; --k) stack.push_back(cc.child[k]);
            }
        }
    }
    const int64_t ng = (int64_t)ws.group_cell.size();
    ws.group_begin.resize(ng + 1);
    for (int64_t g = 0; g < ng; ++g) ws.group_begin[g] = ws.cells[ws.group_cell[g]].begin;
    ws.group_begin[ng] = n;

    // Walks.
    std::vector<std::vector<int32_t>> lep(ng), lsp(ng);
    const double inv_theta2 = theta > 0 ? 1.0 / (theta * theta) : 0.0;
#pragma omp parallel
    {
        std::vector<int64_t> stack;
        stack.reserve(1024);
#pragma omp for schedule(dynamic, 4)
        for (int64_t g = 0; g < ng; ++g) {
            const Cell& gc = ws.cells[ws.group_cell[g]];
            std::vector<int32_t>& ep = lep[g];
            std::vector<int32_t>& spl = lsp[g];
            stack.clear();
            stack.push_back(0);
            while (!stack.empty()) {
                int64_t c = stack.back();
                stack.pop_back();
                const Cell& cc = ws.cells[c];
                bool open;
                if (theta <= 0) {
                    open = true;
                } else {
                    double r2 = box_dist2_point(gc.in_lo, gc.in_hi, cc.com);
                    open = r2 <= cc.side * cc.side * inv_theta2 ||
                           box_overlap(gc.out_lo, gc.out_hi, cc.in_lo, cc.in_hi) ||
                           box_overlap(gc.in_lo, gc.in_hi, cc.out_lo, cc.out_hi);
                }
                if (!open) {
                    spl.push_back((int32_t)c);
                } else if (cc.leaf) {
                    for (int64_t i = cc.begin; i < cc.end; ++i) ep.push_back((int32_t)i);
                } else {
                    for (int k = cc.n_child - 1; k >= 0; --k) stack.push_back(cc.child[k]);
                }
            }
        }
    }
    ws.epj_disp.assign(ng + 1, 0);
    ws.spj_disp.assign(ng + 1, 0);
    for (int64_t g = 0; g < ng; ++g) {
        ws.epj_disp[g + 1] = ws.epj_disp[g] + (int64_t)lep[g].size();
        ws.spj_disp[g + 1] = ws.spj_disp[g] + (int64_t)lsp[g].size();
    }
    ws.id_epj.resize(ws.epj_disp[ng]);
    ws.id_spj.resize(ws.spj_disp[ng]);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t g = 0; g < ng; ++g) {
        std::copy(lep[g].begin(), lep[g].end(), ws.id_epj.begin() + ws.epj_disp[g]);
        std::copy(lsp[g].begin(), lsp[g].end(), ws.id_spj.begin() + ws.spj_disp[g]);
        std::vector<int32_t>().swap(lep[g]);
        std::vector<int32_t>().swap(lsp[g]);
    }
}

}  // namespace

extern "C" {

// Builds the tree and every group's interaction lists.  Returns an opaque
// handle (nullptr on bad arguments).  sizes[0..3] receive: number of groups,
// number of cells, total EPJ list entries, total SPJ list entries.
void* pgfh_build(int64_t n, const double* pos, const double* mass, const double* r_search,
                 double theta, int n_leaf_limit, int n_group_limit, int64_t* sizes) {
    if (n <= 0 || !pos || !mass || !r_search || n_leaf_limit < 1 || n_group_limit < 1) return nullptr;
    if (n > (int64_t)0x7fffffff) return nullptr;
    WalkSet* ws = new WalkSet();
    build(*ws, pos, mass, r_search, n, theta, n_leaf_limit, n_group_limit);
    sizes[0] = (int64_t)ws->group_cell.size();
    sizes[1] = (int64_t)ws->cells.size();
    sizes[2] = (int64_t)ws->id_epj.size();
    sizes[3] = (int64_t)ws->id_spj.size();
    return ws;
}

// Copies the build results into caller-owned arrays sized from pgfh_build's
// sizes: order[n], group_begin[ng+1], epj_disp[ng+1], spj_disp[ng+1],
// id_epj[n_epj_entries], id_spj[n_spj_entries], cell_mass[nc], cell_pos[3nc],
// cell_quad[6nc] (xx, yy, zz, xy, xz, yz), cell_level[nc].
void pgfh_fetch(void* h, int64_t* order, int64_t* group_begin, int64_t* epj_disp, int64_t* spj_disp,
                int32_t* id_epj, int32_t* id_spj, double* cell_mass, double* cell_pos, double* cell_quad,
                int32_t* cell_level) {
    WalkSet* ws = (WalkSet*)h;
    std::memcpy(order, ws->order.data(), sizeof(int64_t) * ws->order.size());
    std::memcpy(group_begin, ws->group_begin.data(), sizeof(int64_t) * ws->group_begin.size());
    std::memcpy(epj_disp, ws->epj_disp.data(), sizeof(int64_t) * ws->epj_disp.size());
    std::memcpy(spj_disp, ws->spj_disp.data(), sizeof(int64_t) * ws->spj_disp.size());
    std::memcpy(id_epj, ws->id_epj.data(), sizeof(int32_t) * ws->id_epj.size());
    std::memcpy(id_spj, ws->id_spj.data(), sizeof(int32_t) * ws->id_spj.size());
    const int64_t nc = (int64_t)ws->cells.size();
    for (int64_t c = 0; c < nc; ++c) {
        const Cell& cc = ws->cells[c];
        cell_mass[c] = cc.mass;
        for (int d = 0; d < 3; ++d) cell_pos[3 * c + d] = cc.com[d];
        for (int k = 0; k < 6; ++k) cell_quad[6 * c + k] = cc.quad[k];
        cell_level[c] = cc.level;
    }
}

void pgfh_free(void* h) { delete (WalkSet*)h; }

}  // extern "C"
