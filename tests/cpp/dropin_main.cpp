// A program written against the reference's FluidSolver surface (the shape of
// 4-solid-boundaries/Fluid.cpp:919-965), compiled against include/ifluids.hpp.
// Prints per step: PCG iterations and the sum of the density field.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ifluids.hpp"

using namespace ifluids;

int main(int argc, char **argv) {
    const int sizeX = argc > 1 ? std::atoi(argv[1]) : 64;
    const int sizeY = argc > 2 ? std::atoi(argv[2]) : 64;
    const int steps = argc > 3 ? std::atoi(argv[3]) : 4;
    const double density = 0.1;
    const double timestep = 0.005;

    std::vector<SolidBody *> bodies;
    bodies.push_back(new SolidBox(0.5, 0.6, 0.7, 0.1, M_PI * 0.25, 0.0, 0.0, 0.0));
    std::vector<const SolidBody *> cBodies(bodies.begin(), bodies.end());

    FluidSolver solver(sizeX, sizeY, density, cBodies);
    for (int i = 0; i < steps; i++) {
        solver.addInflow(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 3.0);
        solver.update(timestep);
        for (SolidBody *b : bodies) b->update(timestep);
        std::vector<double> d = solver.read(IFL_FIELD(IFL_Q_D, IFL_A_SRC));
        double sum = 0.0;
        for (double v : d) sum += v;
        std::printf("%d %.17g\n", solver.stats().pressure.iterations, sum);
    }
    for (SolidBody *b : bodies) delete b;
    return 0;
}
