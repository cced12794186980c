// ref_gpblocks_harness.cpp -- runs the reference's own CPU stepper
// (GrossPitaevskii/GPBlocks.cpp:451-609, integrateInTime) and records golden data.
//
// TEST INFRASTRUCTURE ONLY.  Linked against the unmodified reference sources by
// oracle/build_ref.sh (main renamed, std::max forced in); the product never
// links it.  Output (binary, little endian), consumed by
// tests/golden/make_golden.py:
//   int32  X, Y, Z, V, deg, steps_per_iteration, iterations
//   double lapfac*dt, lapfac0*dt, g*dt, volume, dt
//   int64  lapind[V*deg]
//   double psi0[2*vsize], pot_dt[vsize], even0[2*vsize], odd0[2*vsize]
//   double normsq_error[2*(iterations+1)]   (parsed from the reference's stdout)
// The set-up arrays restate GPBlocks.cpp:455-523 so that the oracle can start
// from the same state; the normsq/error lines come from the reference run itself.
#include "GrossPitaevskii/VortexState.hpp"
#include "Types/Complex.hpp"
#include "Types/Buffer.hpp"
#include "Types/Random.hpp"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

// Symbols defined by the reference translation unit GPBlocks.cpp.
uint integrateInTime(const VortexState& state, const ddouble block_scale, const Vector3& minp, const Vector3& maxp,
                     const uint iteration_period, const uint number_of_iterations);
ddouble potentialRZ(const ddouble r, const ddouble z);
ddouble potentialV3(const Vector3& p);
void getPositions(Buffer<Vector3>& pos);
ddouble getLaplacian(Buffer<uint>& ind, const uint nx, const uint ny, const uint nz);
// GPBlocks.cpp:377-378 defines these with internal linkage; restated here.
static const Vector3 BLOCK_WIDTH = sqrt(8.0) * Vector3(1, 1, 1);
static const ddouble VOLUME = sqrt(32.0 / 9.0);

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s out.bin [kappa g bs half iters vortex_iters]\n", argv[0]);
        return 2;
    }
    const uint kappa = argc > 2 ? (uint)std::atoi(argv[2]) : 1;
    const ddouble g = argc > 3 ? std::atof(argv[3]) : 40.0;
    const ddouble bs = argc > 4 ? std::atof(argv[4]) : 0.2;
    const ddouble half = argc > 5 ? std::atof(argv[5]) : 3.0;
    const uint iters = argc > 6 ? (uint)std::atoi(argv[6]) : 2;
    const uint vortex_iters = argc > 7 ? (uint)std::atoi(argv[7]) : 400;

    VortexState state;
    state.setKappa(kappa);
    state.setG(g);
    state.setRange(0.0, half + 1.0, half + 1.0, 0.1, 0.1);
    state.iterateSolution(potentialRZ, vortex_iters, 1e-29);

    const Vector3 minp(-half, -half, -half), maxp(half, half, half);
    const uint period = 1;

    // --- restatement of the set-up, GPBlocks.cpp:455-523 ---
    const Vector3 dom = maxp - minp;
    const uint xsize = uint(dom.x / (bs * BLOCK_WIDTH.x)) + 1;
    const uint ysize = uint(dom.y / (bs * BLOCK_WIDTH.y)) + 1;
    const uint zsize = uint(dom.z / (bs * BLOCK_WIDTH.z)) + 1;
    const Vector3 p0 = 0.5 * (minp + maxp - bs * Vector3(BLOCK_WIDTH.x * xsize, BLOCK_WIDTH.y * ysize, BLOCK_WIDTH.z * zsize));
    Buffer<Vector3> bpos;
    getPositions(bpos);
    const uint bsize = bpos.size();
    const uint bxsize = (xsize + 1) * bsize;
    const uint bxysize = (ysize + 1) * bxsize;
    const uint ii0 = bxysize + bxsize + bsize;
    const uint vsize = ii0 + (zsize + 1) * bxysize;
    std::vector<double> psi0(2 * (size_t)vsize, 0.0), pot(vsize, 0.0);
    ddouble gg = state.getG();
    ddouble maxpot = 0.0;
    for (uint k = 0; k < zsize; k++)
        for (uint j = 0; j < ysize; j++)
            for (uint i = 0; i < xsize; i++)
                for (uint l = 0; l < bsize; l++) {
                    const uint ii = ii0 + k * bxysize + j * bxsize + i * bsize + l;
                    const Vector3 p(p0.x + bs * (i * BLOCK_WIDTH.x + bpos[l].x), p0.y + bs * (j * BLOCK_WIDTH.y + bpos[l].y),
                                    p0.z + bs * (k * BLOCK_WIDTH.z + bpos[l].z));
                    const Complex c = state.getPsi(p);
                    psi0[2 * (size_t)ii] = c.r;
                    psi0[2 * (size_t)ii + 1] = c.i;
                    pot[ii] = potentialV3(p);
                    const ddouble poti = pot[ii] + gg * c.normsq();
                    if (poti > maxpot) maxpot = poti;
                }
    Buffer<uint> lapind;
    ddouble lapfac = -0.5 * getLaplacian(lapind, bsize, bxsize, bxysize) / (bs * bs);
    const uint lapsize = lapind.size() / bsize;
    ddouble lapfac0 = lapsize * (-lapfac);
    const uint steps = uint(period * (maxpot + lapfac0)) + 1;
    const ddouble dt = period / ddouble(steps);
    gg *= dt;
    lapfac *= dt;
    lapfac0 *= dt;
    for (uint i = 0; i < vsize; i++) pot[i] *= dt;
    std::vector<double> even(2 * (size_t)vsize), odd(2 * (size_t)vsize);
    const Complex oddPhase = state.getPhase(-0.5 * dt);
    Random rnd(54363);
    for (uint i = 0; i < vsize; i++) {
        const Vector2 c = 0.0 * rnd.getUniformCircle();
        const Complex e = Complex(psi0[2 * (size_t)i], psi0[2 * (size_t)i + 1]) * Complex(1.0 + c.x, c.y);
        const Complex o = oddPhase * e;
        even[2 * (size_t)i] = e.r;
        even[2 * (size_t)i + 1] = e.i;
        odd[2 * (size_t)i] = o.r;
        odd[2 * (size_t)i + 1] = o.i;
    }
    const double volume = bs * bs * bs * VOLUME;

    // --- the reference run; capture its normsq/error prints at full precision ---
    std::ostringstream captured;
    std::streambuf* old = std::cout.rdbuf(captured.rdbuf());
    std::cout.precision(17);
    integrateInTime(state, bs, minp, maxp, period, iters);
    std::cout.rdbuf(old);

    std::vector<double> ne;
    std::istringstream in(captured.str());
    std::string line;
    while (std::getline(in, line)) {
        double a, b;
        if (std::sscanf(line.c_str(), "normsq=%lf error=%lf", &a, &b) == 2) {
            ne.push_back(a);
            ne.push_back(b);
        }
    }
    if (ne.size() != 2 * (size_t)(iters + 1)) {
        std::fprintf(stderr, "unexpected reference output:\n%s\n", captured.str().c_str());
        return 1;
    }

    std::ofstream f(argv[1], std::ios::binary);
    const int32_t hdr[7] = {(int32_t)xsize, (int32_t)ysize, (int32_t)zsize, (int32_t)bsize, (int32_t)lapsize,
                            (int32_t)steps, (int32_t)iters};
    f.write((const char*)hdr, sizeof hdr);
    const double sc[5] = {lapfac, lapfac0, gg, volume, dt};
    f.write((const char*)sc, sizeof sc);
    std::vector<int64_t> li(lapind.size());
    for (uint i = 0; i < lapind.size(); i++) li[i] = (int64_t)(int32_t)lapind[i];  // uint wrap-around -> signed offset
    f.write((const char*)li.data(), li.size() * sizeof(int64_t));
    f.write((const char*)psi0.data(), psi0.size() * sizeof(double));
    f.write((const char*)pot.data(), pot.size() * sizeof(double));
    f.write((const char*)even.data(), even.size() * sizeof(double));
    f.write((const char*)odd.data(), odd.size() * sizeof(double));
    f.write((const char*)ne.data(), ne.size() * sizeof(double));
    std::printf("ok %u x %u x %u cells, %u nodes/cell, %u steps/iteration, %u iterations\n", xsize, ysize, zsize, bsize,
                steps, iters);
    return 0;
}
