// GpuPacking (rampack_gb300/host/GpuPacking.hpp) driven like the reference's own Packing
// tests (test/unit_tests/core/PackingTest.cpp:86-166): hard spheres r = 0.25 at three
// positions in a 5x5x5 box.  Prints "ok" and exits 0 when every check holds.
#include <cmath>
#include <limits>
#include <cstdio>
#include <string>
#include <vector>

#include "../../rampack_gb300/host/GpuPacking.hpp"

using rampack_gb300::GpuPacking;

// Stand-ins with the reference's accessors: Vector<3> (operator[]), Matrix<3, 3>
// (operator()(i, j)), ActiveDomain (getBoundsForCoordinate) and an exception type that is not
// std::runtime_error, as the reference side instantiates BasicGpuPacking.
struct RefVector {
    double v[3];
    double operator[](std::size_t i) const { return v[i]; }
};
struct RefMatrix {
    double m[3][3];
    double operator()(std::size_t i, std::size_t j) const { return m[i][j]; }
};
struct RefDomain {
    struct RegionBounds {
        double beg, end;
    };
    RegionBounds b[3];
    const RegionBounds &getBoundsForCoordinate(std::size_t i) const { return b[i]; }
};
struct RefPrecondition {
    std::string what;
};
struct RaiseRef {
    [[noreturn]] static void raise(const std::string &what, const char *, int) { throw RefPrecondition{what}; }
};
using RefPacking = rampack_gb300::BasicGpuPacking<RefVector, RefMatrix, RefDomain, RaiseRef>;

static int failures = 0;
#define CHECK(cond)                                                        \
    do {                                                                   \
        if (!(cond)) {                                                     \
            std::printf("FAILED line %d: %s\n", __LINE__, #cond);          \
            failures++;                                                    \
        }                                                                  \
    } while (0)

static std::vector<GpuPacking::Shape> three() {
    std::vector<GpuPacking::Shape> s(3);
    s[0].position = {0.5, 0.5, 0.5};
    s[1].position = {4.5, 0.5, 0.5};
    s[2].position = {2.5, 2.5, 4.0};
    return s;
}

int main(int argc, char **argv) {
    const double inf = std::numeric_limits<double>::infinity();
    GpuPacking::Mat3 box{5, 0, 0, 0, 5, 0, 0, 0, 5};
    {
        GpuPacking pk(box, three(), 0.25);
        CHECK(pk.countTotalOverlaps() == 0);
        GpuPacking::Mat3 b51{2.55, 0, 0, 0, 2.55, 0, 0, 0, 2.55};
        CHECK(pk.tryScaling(b51) == 0);
        auto s = pk.getShapes();
        CHECK(std::fabs(s[1].position[0] - 2.295) < 1e-9);
    }
    {
        GpuPacking pk(box, three(), 0.25);
        GpuPacking::Mat3 b49{2.45, 0, 0, 0, 2.45, 0, 0, 0, 2.45};
        CHECK(pk.tryScaling(b49) == inf);
        pk.revertScaling();
        auto s = pk.getShapes();
        CHECK(s[2].position[2] == 4.0);
        CHECK(pk.getBox()[0] == 5.0);
    }
    {
        GpuPacking pk(box, three(), 0.25);
        CHECK(pk.tryTranslation(2, {0.01, 0.01, 0.01}) == 0);
        auto s = pk.getShapes();
        CHECK(s[2].position[0] == 2.5);  // tried, not accepted
        pk.acceptTranslation();
        s = pk.getShapes();
        CHECK(s[2].position[0] == 2.51 && s[2].position[2] == 4.01);
        // a rotation by pi/2 about z changes the orientation only
        CHECK(pk.tryRotation(0, {0, -1, 0, 1, 0, 0, 0, 0, 1}) == 0);
        pk.acceptRotation();
        s = pk.getShapes();
        CHECK(s[0].orientation[1] == -1.0 && s[0].position[0] == 0.5);
    }
    {
        // the reference's own types; a translation across a cell face with no ActiveDomain
        // (the reference's serial path) is evaluated as the reference evaluates it, and the
        // same translation with a domain it leaves is rejected before any overlap test
        RefPacking pk(box, three(), 0.25);
        CHECK(pk.tryTranslation(0, RefVector{{0.0, 0.0, 1.3}}) == 0);
        pk.acceptTranslation();
        auto s = pk.getShapes();
        CHECK(s[0].position[2] == 1.8);
        RefDomain dom{{{0.0, 0.5}, {0.0, 0.5}, {0.0, 0.5}}};
        CHECK(pk.tryTranslation(1, RefVector{{0.0, 0.0, 0.1}}, dom) == inf);  // x = 4.5 is outside
        CHECK(pk.tryMove(0, RefVector{{0.01, 0.0, 0.0}}, RefMatrix{{{0, -1, 0}, {1, 0, 0}, {0, 0, 1}}}, dom) == 0);
        pk.acceptMove();
        s = pk.getShapes();
        CHECK(s[0].position[0] == 0.51 && s[0].orientation[1] == -1.0);
        // the tried move puts two spheres 0.29 apart (r = 0.25): an overlap
        CHECK(pk.tryTranslation(2, RefVector{{-1.7, -2.0, -2.2}}) == inf);
        bool raised = false;
        try {
            pk.tryTranslation(3, RefVector{{0, 0, 0}});
        } catch (const RefPrecondition &e) {
            raised = e.what.find("out of range") != std::string::npos;
        }
        CHECK(raised);
        CHECK(pk.tryTranslation(2, RefVector{{0.1, 0.0, 0.0}}) == 0);
        pk.acceptTranslation();
        raised = false;
        try {
            pk.acceptTranslation();  // nothing left to accept
        } catch (const RefPrecondition &) {
            raised = true;
        }
        CHECK(raised);
        s = pk.getShapes();
        CHECK(s[2].position[0] == 2.6 && s[2].position[2] == 4.0);
    }
    {
        // spherocylinders: a device sweep keeps the packing overlap-free
        std::vector<GpuPacking::Shape> sc;
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < 6; j++)
                for (int k = 0; k < 6; k++) {
                    GpuPacking::Shape s;
                    s.position = {1.2 * (i + 0.5), 1.2 * (j + 0.5), 3.6 * (k + 0.5)};
                    sc.push_back(s);
                }
        GpuPacking pk({7.2, 0, 0, 0, 7.2, 0, 0, 0, 21.6}, sc, 0.5, 2.0);
        auto st = pk.performMoves(0.2, 0.2, 42, 0);
        CHECK(st.moves == 2 * sc.size());
        CHECK(st.accepted > 0 && st.accepted < st.moves);
        CHECK(pk.countTotalOverlaps(true) == 0);
        // Packing::store / restore through a RAMSNAP file, and a trajectory recorded while
        // the packing keeps moving
        const std::string dir = argc > 1 ? argv[1] : ".";
        const std::vector<GpuPacking::Shape> before = pk.getShapes();
        pk.store(dir + "/sc.ramsnap", {{"cycles", "1"}});
        {
            rampack_gb300::RamtrjRecorder rec(dir + "/sc.ramtrj", sc.size(), 1);
            rec.recordSnapshot(pk, 1);
            pk.performMoves(0.2, 0.2, 42, 1);
            rec.recordSnapshot(pk, 2);
            rec.close();
        }
        auto aux = pk.restore(dir + "/sc.ramsnap");
        CHECK(aux.size() == 1 && aux["cycles"] == "1");
        const std::vector<GpuPacking::Shape> after = pk.getShapes();
        bool same = true;
        for (std::size_t i = 0; i < sc.size(); i++)
            for (int k = 0; k < 3; k++) same = same && after[i].position[k] == before[i].position[k];
        CHECK(same);
        int64_t np = 0, snaps = 0, step = 0;
        int32_t ver = 0;
        CHECK(rp_ramtrj_info((dir + "/sc.ramtrj").c_str(), &np, &snaps, &step, &ver) == RP_OK);
        CHECK(np == static_cast<int64_t>(sc.size()) && snaps == 2 && step == 1 && ver == 0x101);
    }
    {
        // the calls a Simulation backend makes: overlap counting, rototranslation sweeps, walls.
        // Spherocylinders along x (length 2, radius 0.5) 3.1 apart along x and 0.95 apart
        // across: every side-by-side neighbour pair overlaps.
        std::vector<GpuPacking::Shape> sc;
        for (int i = 0; i < 5; i++)
            for (int j = 0; j < 5; j++)
                for (int k = 0; k < 5; k++) {
                    GpuPacking::Shape s;
                    s.position = {3.1 * (i + 0.5), 0.95 * (j + 0.5), 0.95 * (k + 0.5)};
                    sc.push_back(s);
                }
        GpuPacking pk({15.5, 0, 0, 0, 4.75, 0, 0, 0, 4.75}, sc, 0.5, 2.0);
        pk.toggleOverlapCounting(true);
        const std::size_t n0 = pk.getCachedNumberOfOverlaps();
        CHECK(n0 > 0 && n0 == pk.countTotalOverlaps());
        for (uint64_t c = 0; c < 20; c++) {
            auto st = pk.performMoves(0.1, 0.1, 7, c, true);
            CHECK(st.moves == sc.size());
        }
        const std::size_t n1 = pk.getCachedNumberOfOverlaps();
        CHECK(n1 < n0 && n1 == pk.countTotalOverlaps());
        pk.toggleWalls({true, false, false});
        pk.toggleOverlapCounting(true);
        CHECK(pk.getCachedNumberOfOverlaps() == pk.countTotalOverlaps());
        pk.toggleOverlapCounting(false);
        bool raised = false;
        try {
            (void)pk.getCachedNumberOfOverlaps();
        } catch (const std::runtime_error &) {
            raised = true;
        }
        CHECK(raised);  // Packing::getCachedNumberOfOverlaps throws with counting off
    }
    {
        // two bent rods (PolyspherocylinderTraits, two spherocylinders each): an overlap that
        // only the segments find (centres 0.695 apart, inspheres 0.5), and none where only the
        // circumspheres meet (parallel segments 0.56 apart)
        const std::vector<GpuPacking::Centre> rod{{{-0.35, 0, 0}, 0.25, {0.3, 0, 0.15}},
                                                  {{0.35, 0, 0}, 0.25, {0.3, 0, -0.15}}};
        const GpuPacking::Mat3 big{10, 0, 0, 0, 10, 0, 0, 0, 10};
        std::vector<GpuPacking::Shape> a(2), b(2);
        a[0].position = {5, 5, 5};
        a[1].position = {6.3, 5, 5.35};
        b[0].position = {5, 5, 5};
        b[1].position = {5, 5.56, 5};
        GpuPacking pa(big, a, rod, true), pb(big, b, rod, true);
        CHECK(pa.countTotalOverlaps() == 1);
        CHECK(pb.countTotalOverlaps() == 0);
    }
    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
