// A step-8 (FLIP) program written the way 8-flip/Fluid.cpp:1475-1512 drives
// its solver - bodies created first, update() alone (its inflow is built in),
// compiled against include/ifluids.hpp.  Prints per step: the particle count,
// the pressure PCG iterations and the sum of the density field.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ifluids.hpp"

using namespace ifluids;

int main(int argc, char **argv) {
    const int sizeX = argc > 1 ? std::atoi(argv[1]) : 48;
    const int sizeY = argc > 2 ? std::atoi(argv[2]) : 48;
    const int steps = argc > 3 ? std::atoi(argv[3]) : 3;
    const double densityAir = 0.1, densitySoot = 0.25, diffusion = 0.01, timestep = 0.0025;

    std::vector<SolidBody *> bodies;
    bodies.push_back(new SolidBox(0.5, 0.6, 0.7, 0.1, M_PI * 0.25, 0.0, 0.0, 0.0));
    std::vector<const SolidBody *> cBodies(bodies.begin(), bodies.end());

    FluidSolver solver(sizeX, sizeY, densityAir, densitySoot, diffusion, cBodies, IFL_FLIP);
    for (int i = 0; i < steps; i++) {
        solver.update(timestep);
        std::vector<double> d = solver.read(IFL_FIELD(IFL_Q_D, IFL_A_SRC));
        double sum = 0.0;
        for (double v : d) sum += v;
        std::printf("%zu %d %.17g\n", solver.particles(IFL_P_X).size(), solver.stats().pressure.iterations, sum);
    }
    for (SolidBody *b : bodies) delete b;
    return 0;
}
