// Host-layer checks that need no GPU: ConfigReader, lattice tables and the
// inlet waveform of Simulation::getInletVelocity.  Prints "key value" lines
// that tests/test_host_cpp.py compares against the oracle and the fixtures.
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "ConfigReader.h"
#include "LatticeModel.h"
#include "Simulation.h"

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    ConfigReader cr(argv[1]);
    std::map<std::string, double> vals;
    bool ok = cr.readConfigData(vals);
    std::printf("config_ok %d\n", ok ? 1 : 0);
    for (auto& kv : vals) std::printf("config %s %.17g\n", kv.first.c_str(), kv.second);
    std::vector<std::pair<std::string, std::string>> eq;
    cr.readEquations(eq);
    std::printf("equations %zu\n", eq.size());
    for (int Q : {19, 27}) {
        LatticeModel lm(Q);
        for (int q = 0; q < Q; ++q) {
            std::vector<int> c = lm.GetDirection(q);
            std::printf("lattice %d %d %d %d %d %.17g %d\n", Q, q, c[0], c[1], c[2], lm.GetWeight(q),
                        lm.OppositeDirection(q));
        }
        for (auto& p : lm.m_UnkDisNor) std::printf("unknowns %d %zu\n", Q, p.first.size());
    }
    // waveform at the times Iterate() visits (no GPU: the lattice is created lazily)
    SubDomain sd;
    Simulation sim(sd, 1.0, 1.0, 8e-6, false);
    double t = 0.0;
    for (int s = 0; s < 120000; ++s) {
        if (s % 997 == 0 || s == 119999) std::printf("pulse %d %.17g\n", s, sim.getInletVelocity(t, 0.9));
        t += 8e-6;
    }
    return 0;
}
