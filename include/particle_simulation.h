// particle_simulation.h -- drop-in C++ interface of the GB300 SPH step.
//
// Same class name, enums, parameter struct and public methods as
// CUDASPHNEW/particle_simulation.h:13-324, implemented header-only over the C
// ABI of libsph_gb300.so (sph.h).  Differences a caller of the reference will
// notice, all forced by running headless:
//   * there is no OpenGL: the Get*VertexBufferObject() getters return 0; the
//     state is reached with GetDevicePositions() (float4 per particle, device
//     memory) or CopyPositionsToHost();
//   * Create() builds a simulation from parameters and positions of the
//     caller's choosing; Example01() keeps the reference's demo scene;
//   * Init() may be called again and resets the simulation to its initial
//     state (the reference re-allocates and re-uploads, :1882-2005).
// Errors throw std::runtime_error with the reference's message shape
// ("Exception thrown in FILE: ... LINE: ...", util.h:24-39); Advance*()
// catch, print and continue as the reference does (:2112-2116), without its
// system("pause").
#ifndef PARTICLE_SIMULATION_GB300_H
#define PARTICLE_SIMULATION_GB300_H

#include <cmath>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph.h"

typedef unsigned int GLuint;

// particle_simulation.h:17-23
enum ParticleVertexDataIdx { VD_POS_X, VD_POS_Y, VD_POS_Z, VD_NUM_ELEMENTS };

// particle_simulation.h:28-41
enum ParticleSimulationDataIdx {
    SD_MASS,
    SD_DENSITY,
    SD_PRESSURE,
    SD_ACC_X,
    SD_ACC_Y,
    SD_ACC_Z,
    SD_VEL0_X,
    SD_VEL0_Y,
    SD_VEL0_Z,
    SD_ENERGY,
    SD_NUM_ELEMENTS
};

// particle_simulation.h:44-51
enum BoundaryParticleData { BPD_POS_X, BPD_POS_Y, BPD_POS_Z, BPD_DENSITY, BPD_PRESSURE };

class ParticleSimulation {
public:
    ~ParticleSimulation() { release(); }

    // Allocates device memory and uploads the initial particle data (:1882-2005).
    void Init() {
        release();
        check(sph_create(&mParameters, &mOptions, mVertexData.data(), mSimulationData.data(),
                         mHasBoundary ? &mBoundary : nullptr, &mHandle),
              __FILE__, __LINE__);
    }

    // Copies the parameters to the device (:2078-2083).
    void Bind() const {
        if (mHandle) check(sph_bind(mHandle, &mParameters), __FILE__, __LINE__);
    }

    // One physics step (:2085-2117).
    void Advance() { advance(SPH_STEP_PLAIN); }
    // One step of the sub-particles only, a debug path (:2119-2143).
    void AdvanceSubParticles() { advance(SPH_STEP_SUB_ONLY); }
    // One two-scale step (:2145-2182).
    void AdvanceTwoScale() { advance(SPH_STEP_TWO_SCALE); }

    // Debug check of the boundary maps (declared only in the reference, its
    // body is commented out at :2184-2225): verifies the maps were built.
    void Check3DTextures() const {
        if (!mHasBoundary) return;
        unsigned int dims[3];
        check(sph_boundary_dims(&mBoundary, dims), __FILE__, __LINE__);
    }

    GLuint GetGLParticleVertexBufferObject() const { return 0; }
    GLuint GetGLParticleIndexVertexBufferObject() const { return 0; }
    GLuint GetGLSubParticleVertexBufferObject() const { return 0; }
    GLuint GetGLSubParticleIndexVertexBufferObject() const { return 0; }

    unsigned int GetNumParticlesDefault() const { return counts().numParticlesDefault; }
    unsigned int GetNumSubParticles() const { return counts().numSubParticles; }
    unsigned int GetNumSubParticlesRegular() const { return 8 * counts().numParticlesSplit; }
    unsigned int GetNumSubParticlesBoundary() const { return 8 * counts().numParticlesBoundary; }

    // (3V/(4 pi N))^(1/3) (:2227-2231)
    float GetParticleRadius() const {
        return std::pow((float)((3.0 * mParameters.fluidVolume) / (4.0 * M_PI_GB300 * mParameters.numParticles)),
                        1.0f / 3.0f);
    }
    float GetSubParticleRadius() const { return 0.5f * GetParticleRadius(); }

    // Host copy of the particle states, valid until the next call (:2238-2243).
    const char* GetParticleState() const {
        mStates.resize(mParameters.numParticles);
        check(sph_read(mHandle, SPH_FIELD_STATE, mStates.data(), mStates.size()), __FILE__, __LINE__);
        return mStates.data();
    }

    unsigned int GetNumParticles() const { return mParameters.numParticles; }
    unsigned int GetNumTimesSteps() const { return counts().numTimeSteps; }

    // Keyboard hooks of the reference (:2255-2276): change a parameter, re-Bind.
    void SetNPartThresh(float dVal) {
        mParameters.nPartTresh += dVal;
        std::printf("# particle thresh %f\n", mParameters.nPartTresh);
        Bind();
    }
    void IncreaseCmDistanceThresh() {
        mLeftI = mParameters.cmDistanceThresh;
        mParameters.cmDistanceThresh = 0.5f * (mRightI - mLeftI);
        std::printf("cmDistance = %f\n", mParameters.cmDistanceThresh);
        Bind();
    }
    void DecreaseCmDistanceThresh() {
        mRightI = mParameters.cmDistanceThresh;
        mParameters.cmDistanceThresh = 0.5f * (mRightI - mLeftI);
        std::printf("cmDistance = %f\n", mParameters.cmDistanceThresh);
        Bind();
    }

    // Text dump of the sorted ids, hashes and cell start/end (:2709-2783).
    void SaveInfoTable(const std::string& filename) {
        const unsigned int n = mParameters.numParticles;
        const int cells = mParameters.gridDim[0] * mParameters.gridDim[1] * mParameters.gridDim[2];
        std::vector<int> ids(n), hash(n), start(cells), end(cells);
        check(sph_read_cells(mHandle, 0, hash.data(), ids.data(), start.data(), end.data()), __FILE__, __LINE__);
        std::ofstream file(filename.c_str());
        file << "Number of particles " << n << std::endl;
        file << std::setw(8) << "index" << std::setw(12) << " id" << std::setw(12) << " hash" << std::setw(12)
             << " start" << std::setw(12) << " end" << std::endl;
        for (int i = 0; i < cells; i++) {
            file << std::setw(8) << i;
            if ((unsigned int)i < n) file << std::setw(12) << ids[i] << std::setw(12) << hash[i];
            else file << std::setw(12) << "" << std::setw(12) << "";
            if (start[i] == -1) file << std::setw(12) << "";
            else file << std::setw(12) << start[i];
            if (end[i] == -1) file << std::setw(12) << "" << std::endl;
            else file << std::setw(12) << end[i] << std::endl;
        }
    }

    // Text dump of position, density, pressure and acceleration (:2785-2852).
    void SaveParticleInfo(const std::string& filename) {
        const unsigned int n = mParameters.numParticles;
        std::vector<float> vd((size_t)n * VD_NUM_ELEMENTS), sd((size_t)n * SD_NUM_ELEMENTS);
        check(sph_read(mHandle, SPH_FIELD_VERTEX_DATA, vd.data(), vd.size() * sizeof(float)), __FILE__, __LINE__);
        check(sph_read(mHandle, SPH_FIELD_SIMULATION_DATA, sd.data(), sd.size() * sizeof(float)), __FILE__,
              __LINE__);
        std::ofstream file(filename.c_str());
        const int w = 20;
        const char* head[] = {"Index", "X", "Y", "Z", "Density", "Pressure", "Acc X", "Acc Y", "Acc Z"};
        for (const char* h : head) file << std::setw(w) << h;
        file << std::endl;
        for (unsigned int i = 0; i < n; i++) {
            file << std::setw(w) << i;
            for (int k = 0; k < 3; k++) file << std::setw(w) << vd[(size_t)VD_NUM_ELEMENTS * i + k];
            const int cols[] = {SD_DENSITY, SD_PRESSURE, SD_ACC_X, SD_ACC_Y, SD_ACC_Z};
            for (int c : cols) file << std::setw(w) << sd[(size_t)SD_NUM_ELEMENTS * i + c];
            file << std::endl;
        }
    }

    // Device memory the simulation holds, in bytes (declared only in the
    // reference, :167): not tracked, returns 0.
    unsigned int GetSizeMemoryGPU() const { return 0; }

    // The reference's demo scene (:1745-1817): a 34^3 particle cube dropped in
    // a box container whose walls are the "SPH in complex shapes" maps.
    static ParticleSimulation* Example01() {
        ParticleSimulation* sim = new ParticleSimulation();
        const unsigned int num = (unsigned int)std::pow(40000.0, 1.0 / 3.0);
        const unsigned int n = num * num * num;
        sim->mVertexData.resize((size_t)n * VD_NUM_ELEMENTS);
        sim->mSimulationData.assign((size_t)n * SD_NUM_ELEMENTS, 0.0f);
        const float dx = 0.5f / (float)(num - 1);
        for (unsigned int k = 0; k < num; k++)
            for (unsigned int j = 0; j < num; j++)
                for (unsigned int i = 0; i < num; i++) {
                    size_t idx = (size_t)VD_NUM_ELEMENTS * (num * (num * k + j) + i);
                    sim->mVertexData[idx + VD_POS_X] = -0.65f + i * dx;
                    sim->mVertexData[idx + VD_POS_Y] = -0.45f + j * dx;
                    sim->mVertexData[idx + VD_POS_Z] = -0.25f + k * dx;
                }
        SimulationParameters& p = sim->mParameters;
        std::memset(&p, 0, sizeof(p));
        p.numParticles = n;
        p.kernelParticles = 20;
        p.restDensity = 998.648f;
        p.particleMass = p.restDensity * 0.5f * 0.5f * 0.5f / static_cast<float>(n);
        p.subParticleMass = p.particleMass / 8.0f;
        p.gasStiffness = 3.0f;
        p.dynamicViscosity = 3.0f;
        p.gravity = 9.81f;
        p.tensionCoefficient = 0.0728f;
        p.normThresh = 15.065f;
        const float h = std::pow((float)((3.0f * 0.5f * 0.5f * 0.5f * p.kernelParticles) / (4.0f * M_PI_GB300 * n)),
                                 1.0f / 3.0f);
        setKernels(p, h);
        p.timeStep = 0.003f;
        p.timeStepSubParticles = 0.001f;
        setDomain(p, -1.0f, -1.0f, -1.0f, 1.0f, 1.0f, 1.0f, h, h / 2.0f);
        p.fluidVolume = 0.5f * 0.5f * 0.5f;
        p.restitution = 0.0f;
        p.boxDim[0] = 0.7f;
        p.boxDim[1] = 0.5f;
        p.boxDim[2] = 0.3f;
        p.cmDistanceThresh = 0.5f;
        p.nPartTresh = 20.0f;
        sph_default_options(&sim->mOptions);
        // setUpSphInComplexShapes (:2592-2612)
        sph_boundary_desc& b = sim->mBoundary;
        std::memset(&b, 0, sizeof(b));
        const float s[3] = {-0.8f, -0.6f, -0.4f}, e[3] = {0.8f, 0.6f, 0.4f};
        for (int a = 0; a < 3; a++) {
            b.gridStart[a] = s[a];
            b.gridEnd[a] = e[a];
        }
        b.gridSpacing = h / 4.0f;
        b.restDistance = h;
        b.compactSupport = h;
        b.particleMass = p.particleMass;
        b.restDensity = p.restDensity;
        b.viscosity = p.dynamicViscosity;
        b.particleSpacing = std::pow(p.particleMass / p.restDensity, 1.0f / 3.0f);
        b.numShapes = 1;
        b.shapes[0].kind = SPH_SHAPE_BOX;
        const float box[6] = {0.0f, 0.0f, 0.0f, 0.7f, 0.5f, 0.3f};
        for (int k = 0; k < 6; k++) b.shapes[0].p[k] = box[k];
        sim->mHasBoundary = true;
        return sim;
    }

    // A simulation of the caller's own scene: parameters, initial positions
    // (float[numParticles*3]), optional velocities, options and boundary.
    static ParticleSimulation* Create(const SimulationParameters& params, const float* positions,
                                      const float* velocities = nullptr, const sph_options* options = nullptr,
                                      const sph_boundary_desc* boundary = nullptr) {
        ParticleSimulation* sim = new ParticleSimulation();
        sim->mParameters = params;
        const size_t n = params.numParticles;
        sim->mVertexData.assign(positions, positions + n * VD_NUM_ELEMENTS);
        sim->mSimulationData.assign(n * SD_NUM_ELEMENTS, 0.0f);
        if (velocities)
            for (size_t i = 0; i < n; i++)
                for (int a = 0; a < 3; a++) sim->mSimulationData[i * SD_NUM_ELEMENTS + SD_VEL0_X + a] = velocities[3 * i + a];
        if (options) sim->mOptions = *options;
        else sph_default_options(&sim->mOptions);
        if (boundary) {
            sim->mBoundary = *boundary;
            sim->mHasBoundary = true;
        }
        return sim;
    }

    // Surface particles of the state that entered the last step (:1819-1839;
    // the reference never fills its list): fewer than nPartTresh neighbours
    // or a neighbour centre of mass farther than cmDistanceThresh * h.  All
    // zeros before the first step.
    static int* CreateIsParticleSurfaceList(const ParticleSimulation* sim) {
        const unsigned int n = sim->mParameters.numParticles;
        int* list = new int[n];
        std::memset(list, 0, sizeof(int) * n);
        if (sim->mHandle && sim->counts().numTimeSteps > 0)
            check(sph_surface_particles(sim->mHandle, list), __FILE__, __LINE__);
        int extracted = 0;
        for (unsigned int i = 0; i < n; i++) extracted += list[i];
        std::printf("%d of %d extracted\n", extracted, n);
        return list;
    }

    static void FreeIsParticleSurfaceList(int** list) {
        if (*list == nullptr) return;
        delete[] * list;
        *list = nullptr;
    }

    // -- additions of the headless build --------------------------------
    // float4 per particle (x, y, z, unused) in device memory.
    const float* GetDevicePositions() const {
        void* p = nullptr;
        check(sph_device_pointer(mHandle, 0, &p), __FILE__, __LINE__);
        return static_cast<const float*>(p);
    }
    void CopyPositionsToHost(float* dst) const {
        check(sph_read(mHandle, SPH_FIELD_VERTEX_DATA, dst, sizeof(float) * 3 * (size_t)mParameters.numParticles),
              __FILE__, __LINE__);
    }
    sph_handle Handle() const { return mHandle; }
    SimulationParameters& Parameters() { return mParameters; }

private:
    static constexpr double M_PI_GB300 = 3.14159265358979323846;

    ParticleSimulation() {
        std::memset(&mParameters, 0, sizeof(mParameters));
        sph_default_options(&mOptions);
        std::memset(&mBoundary, 0, sizeof(mBoundary));
    }
    ParticleSimulation(const ParticleSimulation&);
    ParticleSimulation& operator=(const ParticleSimulation&);

    static void check(sph_status st, const char* file, int line) {
        if (st == SPH_OK) return;
        std::string msg = sph_last_error();
        if (msg.empty()) msg = std::string("Exception thrown in FILE: ") + file + " LINE: " + std::to_string(line) +
                               "\nError Message: " + sph_status_string(st) + "\n";
        throw std::runtime_error(msg);
    }

    void advance(int mode) {
        try {
            check(sph_step(mHandle, mode), __FILE__, __LINE__);
        } catch (std::runtime_error& e) {
            std::cout << e.what() << std::endl;
        }
    }

    sph_counts counts() const {
        sph_counts c;
        std::memset(&c, 0, sizeof(c));
        if (mHandle) check(sph_get_counts(mHandle, &c), __FILE__, __LINE__);
        return c;
    }

    void release() {
        if (mHandle) sph_destroy(mHandle);
        mHandle = nullptr;
    }

    // kernel coefficients as Example01 forms them (:1777-1788)
    static void setKernels(SimulationParameters& p, float h) {
        p.compactSupport = h;
        p.compactSupportSub = h / 2.0f;
        p.poly6 = 315.0f / (64.0f * M_PI_GB300 * h * h * h * h * h * h * h * h * h);
        p.gradPoly6 = -945.0f / (32.0f * M_PI_GB300 * h * h * h * h * h * h * h * h * h);
        p.laplPoly6 = -945.0f / (32.0f * M_PI_GB300 * h * h * h * h * h * h * h * h * h);
        p.gradSpiky = -45.0f / (M_PI_GB300 * h * h * h * h * h * h);
        p.laplVisc = 45.0f / (M_PI_GB300 * h * h * h * h * h * h);
        p.poly6Sub = p.poly6 * 512.0f;
        p.gradPoly6Sub = p.gradPoly6 * 512.0f;
        p.laplPoly6Sub = p.laplPoly6 * 512.0f;
        p.gradSpikySub = p.gradSpiky * 64.0f;
        p.laplViscSub = p.laplVisc * 64.0f;
    }

    // set_simulation_domain (:2919-2941)
    static void setDomain(SimulationParameters& p, float xs, float ys, float zs, float xe, float ye, float ze,
                          float spacing, float spacingSub) {
        p.gridOrigin[0] = xs;
        p.gridOrigin[1] = ys;
        p.gridOrigin[2] = zs;
        p.gridDim[0] = static_cast<int>((xe - xs) / spacing + 0.5);
        p.gridDim[1] = static_cast<int>((ye - ys) / spacing + 0.5);
        p.gridDim[2] = static_cast<int>((ze - zs) / spacing + 0.5);
        p.gridDimSubParticles[0] = static_cast<int>((xe - xs) / spacingSub + 0.5);
        p.gridDimSubParticles[1] = static_cast<int>((ye - ys) / spacingSub + 0.5);
        p.gridDimSubParticles[2] = static_cast<int>((ze - zs) / spacingSub + 0.5);
        p.gridSpacing = spacing;
        p.gridSpacingSubParticles = spacingSub;
    }

    SimulationParameters mParameters;
    sph_options mOptions;
    sph_boundary_desc mBoundary;
    bool mHasBoundary = false;
    std::vector<float> mVertexData;
    std::vector<float> mSimulationData;
    mutable std::vector<char> mStates;
    float mLeftI = 0.0f, mRightI = 1.0f;
    sph_handle mHandle = nullptr;
};

#endif  // PARTICLE_SIMULATION_GB300_H
