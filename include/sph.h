/*
 * sph.h -- C ABI of the GB300 SPH step (libsph_gb300.so).
 *
 * This is the thin C layer under the drop-in C++ class `ParticleSimulation`
 * (include/particle_simulation.h), which keeps the public interface of
 * CUDASPHNEW/particle_simulation.h.  Each entry point names the reference
 * interface it replaces.  All pointers are plain host pointers unless a name
 * says "device"; sizes are element counts unless a name says "bytes".
 *
 * Threading: one handle is not thread-safe (as the reference's object is not);
 * distinct handles are independent (parameters live per handle, not in one
 * global __constant__ symbol as at particle_simulation.cu:26).
 *
 * Asynchrony: sph_step() only enqueues work on the handle's stream.  Device-side
 * errors (a particle hashed outside the cell grid, a bounded device wait that
 * gave up) are latched in a device status word and reported by the next
 * sph_synchronize() or sph_read*() call on that handle.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 1

/* Byte-identical to the reference's struct (particle_simulation.h:54-111). */
#ifndef SPH_SIMULATION_PARAMETERS_DEFINED
#define SPH_SIMULATION_PARAMETERS_DEFINED
struct SimulationParameters {
    float gridOrigin[3];
    float gridSpacing;
    int gridDim[3];
    float gridSpacingSubParticles;
    int gridDimSubParticles[3];
    unsigned int numParticles;
    float compactSupport;
    float compactSupportSub;
    int kernelParticles;
    float timeStep;
    float timeStepSubParticles;
    float particleMass;
    float subParticleMass;
    float gasStiffness;
    float restDensity;
    float dynamicViscosity;
    float gravity;
    float tensionCoefficient;
    float normThresh;
    float fluidVolume;
    float poly6;
    float gradPoly6;
    float laplPoly6;
    float gradSpiky;
    float laplVisc;
    float poly6Sub;
    float gradPoly6Sub;
    float laplPoly6Sub;
    float gradSpikySub;
    float laplViscSub;
    float cmDistanceThresh;
    float nPartTresh;
    float boxDim[3];
    float boxCen[3];
    float restitution;
};
#endif
typedef struct SimulationParameters SimulationParameters;

/* Behaviour the reference hard-codes.  sph_default_options() gives the
 * reference's values. */
typedef struct sph_options {
    int gravityAxis;    /* axis the gravity acts along (negative direction);
                           reference: 1, particle_simulation.cu:471 */
    int boxCollision;   /* 1: collision_handling after integrate in every
                           step (AdvanceTwoScale, :2170); 0: Advance (:2106) */
    int childMode;      /* two-scale children.  0: re-seeded from their parent
                           in every step, as the reference runs
                           (initialize_sub_particles, :1023-1090).  1: kept
                           while the parent stays in its class; seeded when
                           the parent enters the split or boundary class or
                           moves between them (the transitions listed at
                           :1052-1055); a parent leaving the split class
                           first takes its children's mean position and
                           velocity (merge-back, no reference counterpart) */
    int cellRelative;   /* 1: positions are stored relative to the low corner
                           of their grid cell (the cell's integer coordinates
                           beside them), so pair offsets and the integration
                           step keep FP32 precision however far the scene lies
                           from the origin (every position resolves half a
                           unit in the last place of gridSpacing); the
                           reference stores absolute FP32 positions (0).
                           Plain steps only; gridDim at most 2048 x 2048 x
                           1024.  No reference counterpart. */
    float splitMin[3];  /* two-scale split region; reference: 0.2 <= x <= 0.5 */
    float splitMax[3];  /* (find_split_particles, :948) */
    float neighbourSkin; /* plain and learned steps of handles with absolute
                            positions (a batch decides its builds per scene,
                            so a scene builds when it would alone): the neighbour
                            candidates within (1 + neighbourSkin) * compactSupport
                            are recorded when the lists are built and reused by
                            later steps until some particle has moved more than
                            0.45 * neighbourSkin * compactSupport since, when
                            they are built again (a Verlet list; a pair that
                            comes within compactSupport in the meantime was
                            within the skin when they were built).  A step
                            that builds no lists skips the hash, sort and cell
                            tables (sph_read_cells builds that step's tables
                            when asked, bit exact); only the order in which the
                            neighbour sums are taken follows the lists.  0: the
                            neighbour search runs in every step, as the
                            reference does (compute_particle_density_pressure,
                            :196-256).  In [0, 0.4].  No reference counterpart. */
} sph_options;

/* Boundary solids ("SPH in complex shapes", SphInComplexShapes.h:18-93). */
enum {
    SPH_SHAPE_SPHERE = 1, /* p = (cx, cy, cz, r): solid sphere */
    SPH_SHAPE_CONE = 2,   /* p = (bx, by, bz, R, H): solid cone on its base, axis +z */
    SPH_SHAPE_BOX = 3,    /* p = (cx, cy, cz, ex, ey, ez): container, fluid inside
                             (SetBox, SphInComplexShapes.cpp:203-313) */
    SPH_SHAPE_MESH = 4    /* p[0] = index into sph_boundary_desc.sdfGrids: a solid
                             given by a signed distance grid (negative inside),
                             e.g. from sph_sdf_from_mesh; read trilinearly, no
                             solid outside the grid's box */
};

/* A signed distance grid (BoundaryMap, boundary_map.h:35-122): nodes
 * origin + (i, j, k)*dx, x fastest; distance negative inside the solid.
 * Nodes within maxDist = max(restDistance, compactSupport) of the surface
 * hold the exact distance and a unit normal (node minus closest surface
 * point); the others hold +-maxDist and a zero normal (a grid read from the
 * reference's text format holds +restDistance there, as its Load does). */
typedef struct sph_sdf_grid {
    float origin[3];
    float dx;
    unsigned int dims[3];
    float restDistance;
    float compactSupport;
    float maxDist;
    float* distance;    /* float[dims[0]*dims[1]*dims[2]] */
    float* normal;      /* float[3*dims product], or NULL */
} sph_sdf_grid;

typedef struct sph_shape {
    int kind;
    float p[7];
} sph_shape;

/* The arguments of SphInComplexShapes' constructor (SphInComplexShapes.h:21-23)
 * plus the solids.  The maps (signed distance, wall density, wall viscosity)
 * are built on the GPU at sph_create and read trilinearly during the step. */
typedef struct sph_boundary_desc {
    float gridStart[3];
    float gridEnd[3];
    float gridSpacing;
    float restDistance;
    float compactSupport;
    float particleMass;
    float restDensity;
    float viscosity;
    float particleSpacing;
    int numShapes;
    sph_shape shapes[8];
    const sph_sdf_grid* sdfGrids; /* the grids of SPH_SHAPE_MESH solids (host
                                     memory, read during sph_create only) */
    int numSdfGrids;
} sph_boundary_desc;

typedef enum sph_status {
    SPH_OK = 0,
    SPH_ERR_INVALID_ARGUMENT = 1,
    SPH_ERR_CUDA = 2,
    SPH_ERR_OUT_OF_MEMORY = 3,
    SPH_ERR_OUT_OF_DOMAIN = 4, /* a particle hashed outside the cell grid */
    SPH_ERR_DEVICE_WAIT = 5,   /* a bounded device-side wait gave up */
    SPH_ERR_NOT_SUPPORTED = 6,
    SPH_ERR_NON_FINITE = 7     /* a NaN/inf position entered the step */
} sph_status;

typedef enum sph_step_mode {
    SPH_STEP_PLAIN = 0,     /* Advance (particle_simulation.cu:2085-2117) */
    SPH_STEP_TWO_SCALE = 1, /* AdvanceTwoScale (:2145-2182) */
    SPH_STEP_SUB_ONLY = 2,  /* AdvanceSubParticles (:2119-2143) */
    SPH_STEP_LEARNED = 3    /* one plain step of stride*dt plus the learned
                               correction (no reference counterpart; needs a
                               trained or loaded corrector, see below) */
} sph_step_mode;

/* Per-particle fields, returned in particle-index order. */
typedef enum sph_field {
    SPH_FIELD_VERTEX_DATA = 0,     /* float[n*3]  VD layout (particle_simulation.h:17-23) */
    SPH_FIELD_SIMULATION_DATA = 1, /* float[n*10] SD layout (particle_simulation.h:28-41) */
    SPH_FIELD_VELOCITY = 2,        /* float[n*3] */
    SPH_FIELD_ACCELERATION = 3,    /* float[n*3] */
    SPH_FIELD_DENSITY = 4,         /* float[n] */
    SPH_FIELD_PRESSURE = 5,        /* float[n] */
    SPH_FIELD_STATE = 6,           /* char[n] (GetParticleState) */
    /* two-scale pass: child slots 8*parent + k (capacity 8n), lists */
    SPH_FIELD_SUB_VERTEX_DATA = 7,     /* float[8n*3] child positions by slot */
    SPH_FIELD_SUB_SIMULATION_DATA = 8, /* float[8n*10] child SD by slot */
    SPH_FIELD_SUB_IDS = 9,             /* int[numSubParticles] active child slots */
    SPH_FIELD_SPLIT_IDS = 10,          /* int[numParticlesSplit] */
    SPH_FIELD_BOUNDARY_IDS = 11,       /* int[numParticlesBoundary] */
    SPH_FIELD_DEFAULT_IDS = 12         /* int[numParticlesDefault] */
} sph_field;

typedef struct sph_counts {
    unsigned int numParticles;
    unsigned int numParticlesDefault;  /* GetNumParticlesDefault */
    unsigned int numParticlesSplit;
    unsigned int numParticlesBoundary;
    unsigned int numSubParticles;      /* GetNumSubParticles */
    unsigned int numTimeSteps;         /* GetNumTimesSteps */
    unsigned int numCells;
    unsigned int numSubCells;
} sph_counts;

typedef struct sph_sim* sph_handle;

/* Reference defaults for sph_options. */
void sph_default_options(sph_options* opts);

/* Init (particle_simulation.cu:1882-2005) + Bind (:2078-2083): allocates all
 * device memory, uploads the initial vertex data (float[n*3]) and optionally
 * the simulation data (float[n*10], velocities taken from SD_VEL0_*; NULL means
 * zero), and builds the boundary maps when `boundary` is not NULL
 * (setUpSphInComplexShapes, :2592-2683).  n = params->numParticles.
 * `opts` NULL means sph_default_options(). */
sph_status sph_create(const SimulationParameters* params, const sph_options* opts,
                      const float* vertexData, const float* simulationData,
                      const sph_boundary_desc* boundary, sph_handle* out);

/* Batched scenes (no reference counterpart): many independent simulations
 * in one handle, each with its own parameters, particles and (optional)
 * boundary maps.  Every stage of a plain step is one launch over all scenes;
 * the particles of all scenes share one sort over the concatenation of the
 * scenes' cell grids, each scene's cells at its own offset, so a scene's
 * results are bit-identical to running it alone.  Per-particle fields are
 * read and written scene after scene (sph_batch_info gives the ranges).
 * Batched handles take SPH_STEP_PLAIN steps only; sph_bind, the two-scale
 * and learned modes and sph_get_diagnostics answer SPH_ERR_NOT_SUPPORTED.
 * All scenes use the same sph_options (gravity axis, box collision). */
typedef struct sph_scene {
    const SimulationParameters* params; /* numParticles = this scene's count */
    const float* vertexData;            /* float[n*3] */
    const float* simulationData;        /* float[n*10] or NULL */
    const sph_boundary_desc* boundary;  /* or NULL */
} sph_scene;
sph_status sph_create_batch(const sph_scene* scenes, int numScenes, const sph_options* opts,
                            sph_handle* out);
/* Scene k owns particles [firstParticle[k], firstParticle[k+1]) and cells
 * [firstCell[k], firstCell[k+1]) of the handle; either array may be NULL
 * (else numScenes + 1 entries). */
sph_status sph_batch_info(sph_handle h, int* numScenes, unsigned int* firstParticle, unsigned int* firstCell);

/* ~ParticleSimulation (:1691-1743). */
sph_status sph_destroy(sph_handle h);

/* Bind (:2078-2083) with new parameters (SetNPartThresh etc. re-Bind,
 * :2255-2276).  numParticles and the grid dimensions must not change. */
sph_status sph_bind(sph_handle h, const SimulationParameters* params);

/* Runs later work of this handle on `stream` (a cudaStream_t; NULL restores
 * the handle's own stream). */
sph_status sph_set_stream(sph_handle h, void* stream);

/* Advance / AdvanceTwoScale / AdvanceSubParticles: enqueues one step.  The
 * plain step does not run the two-scale bookkeeping (particle states, lists,
 * children): it does not change the coarse particles; the two-scale step
 * does, with its counts kept on the device. */
sph_status sph_step(sph_handle h, int mode);

/* Enqueues `count` steps of `mode` (one CUDA-graph launch each once captured). */
sph_status sph_step_many(sph_handle h, int mode, int count);

/* Waits for the handle's stream; returns the latched device status. */
sph_status sph_synchronize(sph_handle h);

/* Copies a field to host memory (GetParticleState, SaveParticleInfo,
 * :2238-2243, :2785-2852).  `bytes` must be at least the field's size.
 * Returns when the data is in place.  Positions and velocities bound for a
 * page-locked destination are packed into it by the kernel itself, over the
 * host link; other fields and pageable destinations are gathered into a
 * device staging buffer and copied back by one DMA copy. */
sph_status sph_read(sph_handle h, int field, void* dst, size_t bytes);

/* Overwrites a field from host memory (SPH_FIELD_VERTEX_DATA,
 * SPH_FIELD_VELOCITY or SPH_FIELD_SIMULATION_DATA).  A page-locked source of
 * positions or velocities is read by the unpacking kernel itself, later on
 * the handle's stream (as an asynchronous copy from pinned memory would be);
 * when that stream still has work queued, the upload runs beside it on a
 * stream of its own, into a device buffer that is copied into place on the
 * handle's stream once it has landed, so the host link and the queued work
 * overlap.  Either way: keep the source unchanged until the next
 * synchronising call. */
sph_status sph_write(sph_handle h, int field, const void* src, size_t bytes);

/* sph_read without waiting: enqueues the read of a field of the particle
 * grid (VD, velocity, acceleration, density or pressure) on the handle's
 * stream and returns.  The destination holds the field once the stream has
 * reached that point (sph_synchronize); the conditions steps latch are
 * reported by the next synchronising call.  A loop of sph_write (page-locked
 * sources), sph_step and sph_read_async thus overlaps each step's uploads
 * with the work and read-back queued before them.  No reference
 * counterpart. */
sph_status sph_read_async(sph_handle h, int field, void* dst, size_t bytes);

/* The neighbour-search tables of the last step (SaveInfoTable, :2709-2783):
 * sorted hashes, sorted particle ids (the sort permutation), and the
 * cell start/end lists with 0xFFFFFFFF for empty cells.  level 0 is the
 * particle grid, level 1 the sub-particle grid.  Any pointer may be NULL.
 * After a step over reused neighbour lists that built none (it skips the
 * tables) the level-0 tables are built here from the state that step
 * started from, as the step would have built them. */
sph_status sph_read_cells(sph_handle h, int level, int* sortedHash, int* sortedIds,
                          int* cellStart, int* cellEnd);

/* Particle counts (GetNumParticles*, GetNumSubParticles*, GetNumTimesSteps). */
sph_status sph_get_counts(sph_handle h, sph_counts* out);

/* ---------------------------------------------------------------------------
 * Meshes and signed distance grids (BoundaryMap, PointInMeshTest).
 * ------------------------------------------------------------------------- */
typedef struct sph_mesh {
    float* vertices;        /* float[numVertices*3] */
    unsigned int numVertices;
    unsigned int* faces;    /* uint[numFaces*3], 0-based vertex indices */
    unsigned int numFaces;
} sph_mesh;

/* Reads the `v` and `f` records of a Wavefront OBJ file (TriangleMesh,
 * triangle_mesh.cpp:16-37): f entries may be "i", "i/t", "i//n" or "i/t/n",
 * 1-based or negative (relative); polygons are split into triangle fans.
 * The arrays are malloc'ed: free them with sph_mesh_free. */
sph_status sph_obj_load(const char* path, sph_mesh* out);
void sph_mesh_free(sph_mesh* mesh);

/* BoundaryMap(config) + AddCanvas(mesh) (boundary_map.cpp:25-95, 351-470) on
 * the GPU: a grid over the mesh's bounding box, ceil(extent/dx) + 1 nodes per
 * axis.  sph_sdf_from_mesh_on_grid takes the grid (origin, dx, dims) from
 * the caller instead, e.g. the bounding box grown by a margin so that the
 * grid can serve as an SPH_SHAPE_MESH solid.  The arrays are malloc'ed: free
 * them with sph_sdf_free. */
sph_status sph_sdf_from_mesh(const sph_mesh* mesh, float restDistance, float compactSupport, float dx,
                             sph_sdf_grid* out);
sph_status sph_sdf_from_mesh_on_grid(const sph_mesh* mesh, const float origin[3], float dx,
                                     const unsigned int dims[3], float restDistance,
                                     float compactSupport, sph_sdf_grid* out);
/* The reference's boundary-map text file (BoundaryMap::Save / Load,
 * boundary_map.cpp:161-287): the band's nodes only, one value per line. */
sph_status sph_sdf_save(const sph_sdf_grid* grid, const char* path);
sph_status sph_sdf_load(const char* path, sph_sdf_grid* out);
void sph_sdf_free(sph_sdf_grid* grid);

/* FP64 conservation diagnostics of the coarse particles (no reference
 * counterpart; the reference's SD_ENERGY column, particle_simulation.h:40, is
 * never filled).  mass, momentum and energies are of the current state,
 * potential = sum m*g*x[gravityAxis]; the density terms are of the last
 * density pass (zero before the first step).  Reduced on the GPU in double
 * precision in a fixed order, so repeated calls on one state agree bit for
 * bit.  Synchronises the handle's stream. */
typedef struct sph_diagnostics {
    double mass;
    double momentum[3];
    double kineticEnergy;
    double potentialEnergy;
    double densityMean;
    double densityMaxRelError; /* max |rho - restDensity| / restDensity */
} sph_diagnostics;
sph_status sph_get_diagnostics(sph_handle h, sph_diagnostics* out);

/* ---------------------------------------------------------------------------
 * Learned step corrector (no reference counterpart).
 *
 * A per-particle MLP, 24 neighbour features -> 64 -> 64 -> 6 with SiLU, BF16
 * weights and activations and FP32 accumulation on the tensor cores, corrects
 * one plain step of stride*dt (SPH_STEP_LEARNED) towards `stride` plain steps
 * of dt.  It is trained on the device from the plain solver's own trajectory.
 * The plain solver is the fallback and the arbiter: every auditInterval-th
 * learned step is also run as `stride` plain steps from the same state, and
 * when the largest per-particle relative density difference between the two
 * results exceeds densityTolerance the plain result is kept (a rollback).
 * ------------------------------------------------------------------------- */
#define SPH_CORRECTOR_FEATURES 24
#define SPH_CORRECTOR_OUTPUTS 6
/* Model blob: FP32 weights W1[64][32] (input columns 24..31 zero), W2[64][64],
 * W3[16][64] (rows 6..15 zero), b1[64], b2[64], b3[16] (6..15 zero) -- the
 * first SPH_CORRECTOR_WEIGHTS floats -- then the feature means[24], feature
 * deviations[24], and per output the target mean[6], deviation[6] and scale[6].
 * With a scale s > 0 the network's standardised output y gives the correction
 * s*sinh(mean + deviation*y) (the targets were compressed as asinh(t/s));
 * s <= 0 gives mean + deviation*y. */
#define SPH_CORRECTOR_WEIGHTS 7312
#define SPH_CORRECTOR_FLOATS 7378

typedef struct sph_corrector_config {
    int trainSteps;         /* plain steps of dt that generate samples (2000) */
    int stride;             /* a learned step is stride*dt (4) */
    int epochs;             /* passes over the samples (6) */
    int batchTiles;         /* 128-sample tiles per Adam step (128) */
    float learningRate;     /* Adam, decayed linearly to 1% (2e-3) */
    float densityTolerance; /* audit threshold (0.01) */
    int auditInterval;      /* audit every k-th learned step (16); 0: never */
    unsigned int seed;      /* weight initialisation and sample order */
    float targetScale;      /* > 0: train on asinh(t/s) with s = targetScale x the
                               target's deviation (compresses the heavy tail of
                               the corrections); 0: on t itself (default) */
} sph_corrector_config;

typedef struct sph_corrector_report {
    unsigned int samples;         /* training samples (particles x start states) */
    unsigned int optimizerSteps;
    float firstEpochLoss;         /* mean loss on standardised targets */
    float lastEpochLoss;
    float trainMilliseconds;      /* sample generation + training, device time */
    unsigned int learnedSteps;    /* SPH_STEP_LEARNED steps taken */
    unsigned int audits;
    unsigned int rollbacks;
    float lastAuditError;         /* max relative density difference of the last audit */
    float maxAuditError;
} sph_corrector_report;

void sph_corrector_default_config(sph_corrector_config* cfg);

/* Runs cfg->trainSteps plain steps of dt from the handle's current state (the
 * handle advances), collects (features, correction) samples for every start
 * state with `stride` steps after it, fits the standardisation and trains the
 * MLP with Adam.  Deterministic for a given seed. */
sph_status sph_corrector_train(sph_handle h, const sph_corrector_config* cfg);

/* Replaces the corrector by a model blob (SPH_CORRECTOR_FLOATS floats). */
sph_status sph_corrector_load(sph_handle h, const sph_corrector_config* cfg, const float* model, size_t count);
sph_status sph_corrector_save(sph_handle h, float* model, size_t count);
sph_status sph_corrector_get_report(sph_handle h, sph_corrector_report* out);

/* Checking entry points: corrections (count x 6, denormalised) of given raw
 * features (count x 24), and the loss gradient (SPH_CORRECTOR_WEIGHTS floats,
 * blob order) and summed loss of given samples (targets count
 * x 8, first 6 used), both through the tensor-core kernels. */
sph_status sph_corrector_predict(sph_handle h, const float* features, int count, float* corrections);
sph_status sph_corrector_gradient(sph_handle h, const float* features, const float* targets, int count,
                                  float* grad, float* loss);

/* Feature recording (off by default): while enabled, each SPH_STEP_LEARNED
 * step also writes its particles' input features (24 floats each) to the
 * handle, 96 bytes per particle and step of extra device-memory writes.
 * Needs a trained or loaded corrector.  No reference counterpart. */
sph_status sph_corrector_record_features(sph_handle h, int enable);

/* The corrector's input features (n x 24, particle order) that the last
 * SPH_STEP_LEARNED step taken with recording enabled computed from the state
 * it started from. */
sph_status sph_read_features(sph_handle h, float* dst, size_t bytes);

/* CreateIsParticleSurfaceList (particle_simulation.cu:1818-1839): flags[i] =
 * 1 when particle i, in the state that entered the last step, has fewer
 * than nPartTresh neighbours within compactSupport or its neighbours'
 * centre of mass lies farther than cmDistanceThresh * compactSupport from
 * it (the thresholds of SimulationParameters; the reference never fills its
 * list).  int[n], particle order. */
sph_status sph_surface_particles(sph_handle h, int* flags);  /* not for batched handles */

/* Headless renderer: the sphere imposters of the reference's
 * TwoScaleStateSub renderer (twoscalestatesub.cpp:84-161,
 * twoscalestatesub_{v,g,f}.glsl) splatted by CUDA kernels into an image, no
 * graphics API.  Matrices are column-major, as OpenGL takes them. */
typedef struct sph_camera {
    float view[16];
    float proj[16];
} sph_camera;

/* cgtkGLLookAt (cgtk/src/opengl.c:10-46): the view matrix of an eye looking
 * at centre with the given up vector. */
sph_status sph_camera_look_at(sph_camera* cam, const float eye[3], const float centre[3], const float up[3]);
/* cgtkGLPerspective + cgtkGLFrustum (cgtk/src/opengl.c:48-78). */
sph_status sph_camera_perspective(sph_camera* cam, float fovy, float aspect, float znear, float zfar);

enum {
    SPH_RENDER_PARTICLES = 0,     /* renderLow: every coarse particle, blue */
    SPH_RENDER_TWO_SCALE = 1,     /* render: default particles (blue), regular
                                     (yellow) and boundary (red) sub-particles
                                     at half the radius, in that draw order */
    SPH_RENDER_SUB_PARTICLES = 2  /* renderRegularSubParticles: the
                                     sub-particles alone */
};

/* Renders the current state: particle radius GetParticleRadius()
 * ((3 fluidVolume / (4 pi n))^(1/3), particle_simulation.cu:2227-2236),
 * white background, shading 0.9 + 0.1 max(0, n.z), GL_LESS depth test on a
 * 24-bit depth buffer (the first drawn fragment keeps a tie).  rgba: host
 * uint8[height][width][4], rows top to bottom; depth (optional): host
 * float[height][width], the stored depth in [0, 1] (1 where nothing was
 * drawn).  The two-scale modes need a two-scale step to have run.  At most
 * 2^26 pixels. */
sph_status sph_render(sph_handle h, const sph_camera* cam, int width, int height, int what, unsigned char* rgba,
                      float* depth);

/* PortablePixmap::save's format (portable_pixmap.cpp:23-40): ASCII P3,
 * maximum 255, one value per line, the RGB of `rgba` rows top to bottom. */
sph_status sph_image_save_ppm(const char* path, const unsigned char* rgba, int width, int height);

/* Device pointer of a field in the handle's layout, for zero-copy consumers
 * (replaces the OpenGL VBO getters, :2278-2301): 0 = positions (float4[n],
 * particle order), 1 = velocities (float4[n]). */
sph_status sph_device_pointer(sph_handle h, int which, void** devicePtr);

/* The boundary maps of `desc`, built on the GPU, copied to host grids of
 * dims[0]*dims[1]*dims[2] floats each, x fastest (CreateDistanceTextureData
 * etc., SphInComplexShapes.cpp:366-427).  Any output may be NULL. */
sph_status sph_boundary_dims(const sph_boundary_desc* desc, unsigned int dims[3]);
sph_status sph_boundary_maps(const sph_boundary_desc* desc, float* distance,
                             float* density, float* viscosity);

/* Launch configuration of the step's neighbour kernels.  None of these
 * fields changes a result bit: pruned stencil cells hold no particle within
 * the support radius, and both force forms sum the same terms in the same
 * order.  (kahan selects compensated summation, which does change rounding,
 * and is never altered by the autotuner.)  No reference counterpart: the
 * reference hard-codes 256 threads per block (particle_simulation.cu:2943-2957). */
typedef struct sph_tuning {
    int densityBlock;  /* 64, 128 or 256 */
    int forceBlock;    /* 64, 128 or 256 */
    int forceVariant;  /* 0: direct loop, 1: per-chunk hit mask, then interactions,
                          2: neighbour masks recorded by the density stage,
                          3: as 2, each warp's neighbour rows staged in shared
                          memory (plain handles; batched and cell-relative
                          handles run 2) */
    int prune;         /* 1: cut stencil rows to the half-cells within reach of h */
    int kahan;         /* 1: compensated density and force sums */
} sph_tuning;

sph_status sph_get_tuning(sph_handle h, sph_tuning* out);
sph_status sph_set_tuning(sph_handle h, const sph_tuning* t);

/* Times every candidate launch configuration of the density and force
 * kernels on the handle's current particle state (`reps` launches each, CUDA
 * events on the handle's stream), keeps the fastest and returns it.  The
 * simulation state is left untouched.  No reference counterpart. */
sph_status sph_autotune(sph_handle h, int reps, sph_tuning* chosen);

/* Stage timing with CUDA events on the handle's stream (CudaTimer,
 * util.cpp:6-41, generalised to every stage).  After enabling, each step
 * records events between its stages; sph_stage_times() returns the summed
 * milliseconds and the number of timed steps per stage since the last call
 * and resets them.  Stages (sph_stage_name): 0 hash_count, 1 cell_scan,
 * 2 scatter, 3 rank_gather, 4 density, 5 force_integrate -- every plain and
 * two-scale step -- then, in two-scale steps only, 6 ts_children (states,
 * split lists, children, projection), 7 sub_sort, 8 sub_density, 9 sub_force.
 * An interval holds its stage's launches and the gaps between them. */
sph_status sph_set_stage_timing(sph_handle h, int enable);
sph_status sph_stage_times(sph_handle h, float* ms, int* counts, int capacity, int* numStages);
const char* sph_stage_name(int stage);

/* Average device time of one launch of a stage's kernel (stage 4: density,
 * 5: force; see sph_stage_name), launched `reps` times back to back on the
 * last step's sorted state between two CUDA events on the handle's stream,
 * with the current tuning.  Both kernels rewrite what they wrote: after a
 * plain step the force stage leaves the state that step left (after another
 * kind of step it replaces that step's result with the plain step's).  No
 * reference counterpart. */
sph_status sph_time_kernel(sph_handle h, int stage, int reps, float* microseconds);

/* How many times the handle's plain and learned steps have built their
 * reused neighbour lists (sph_options.neighbourSkin; 0 when the handle has
 * none; a batch: its scenes' builds summed).  Waits for the handle's stream.
 * No reference counterpart. */
sph_status sph_neighbour_builds(sph_handle h, unsigned int* builds);

/* Largest inputs sph_cell_tables_noalloc() accepts. */
#define SPH_NOALLOC_MAX_PARTICLES 65536
#define SPH_NOALLOC_MAX_CELLS 262144

/* The neighbour-search tables of one set of positions -- sorted hashes, the
 * sort permutation, and cell start/end with 0xFFFFFFFF for empty cells, as
 * sph_step() + sph_read_cells() give them -- built without allocating any
 * memory, for callers that cannot call cudaMalloc where they need the tables
 * (a frame loop an allocation would stall, or an application whose device
 * memory is all handed to its own allocator).  No counterpart in the
 * reference; it follows computeParticleHash, sortParticleIdsByHash and
 * computeCellStartEndList (particle_simulation.cu:2320-2369).
 *
 * Inputs and outputs are device pointers the caller owns: devVertexData
 * float[n*3] (the VD layout), devSortedHash and devSortedIds int[n],
 * devCellStart and devCellEnd int[gridDim[0]*gridDim[1]*gridDim[2]].  All
 * intermediate data lives in one fixed device array of about 2.9 MB that the
 * library holds on every GPU it runs on until the process exits; n above
 * SPH_NOALLOC_MAX_PARTICLES or more cells than SPH_NOALLOC_MAX_CELLS are
 * rejected with SPH_ERR_INVALID_ARGUMENT.  Calls share that array: calls whose
 * work overlaps on the GPU race and must be serialised by the caller.  The
 * first call on a device looks the array up for that device; make it before
 * any stream capture on that device.  The call enqueues its work on `stream`
 * (a cudaStream_t, NULL for the default stream) and returns once that work is
 * done; on a stream that is being captured it enqueues nothing and returns
 * SPH_ERR_NOT_SUPPORTED.  A non-finite position gives SPH_ERR_NON_FINITE and
 * one hashed outside the grid SPH_ERR_OUT_OF_DOMAIN; the outputs are then
 * unspecified.  The stable order inside a cell costs k^2 comparisons for a
 * cell of k particles, so positions crowded into a few cells are slow. */
sph_status sph_cell_tables_noalloc(const SimulationParameters* params, const float* devVertexData,
                                   unsigned int n, int* devSortedHash, int* devSortedIds,
                                   int* devCellStart, int* devCellEnd, void* stream);

/* Human-readable message of the last failing call on this thread, in the
 * reference's "Exception thrown in FILE: ... LINE: ..." shape (util.h:24-39). */
const char* sph_last_error(void);
const char* sph_status_string(sph_status s);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */
