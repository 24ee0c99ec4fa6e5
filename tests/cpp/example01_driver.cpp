// Test driver: the reference's main-loop calls (main.cpp:80-82, 148) against
// the drop-in header, headless.  Usage: example01_driver <steps> <out prefix>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "particle_simulation.h"

int main(int argc, char** argv) {
    int steps = argc > 1 ? std::atoi(argv[1]) : 2;
    std::string prefix = argc > 2 ? argv[2] : "example01";
    ParticleSimulation* sim = ParticleSimulation::Example01();
    sim->Init();
    sim->Bind();
    for (int i = 0; i < steps; i++) sim->Advance();
    sim->SaveParticleInfo(prefix + "_particles.txt");
    sim->SaveInfoTable(prefix + "_table.txt");
    std::printf("particles %u steps %u radius %.6f\n", sim->GetNumParticles(), sim->GetNumTimesSteps(),
                sim->GetParticleRadius());
    int* surf = ParticleSimulation::CreateIsParticleSurfaceList(sim);
    ParticleSimulation::FreeIsParticleSurfaceList(&surf);
    delete sim;
    return 0;
}
