// The reference's ten free functions (project/smokeSimulation.cuh:4-17) on top of the C ABI.
//
// Module state mirrors the reference's globals: one implicit simulation, an object registry
// that outlives deleteVolume (smokeSimulation.cu:54-58), and gravity/buoyancy variables whose
// addresses the caller's UI writes through getGravity/getBuoyancy (:28-36, main.cpp:832-833).
// simulate() re-applies the registry and the two variables before every step, so changes made
// between calls take effect on the next step as they do in the reference.  Errors print and
// exit(-1) like the reference's error paths (:132-135, :815-817).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/smoke_gb300.h"
#include "../../include/smokeSimulation_gb300.cuh"

namespace {

struct RefObject {
    int type;  // 0 obstacle, 1 smoke source (Sphere::type, smokeSimulation.cu:50)
    float x, y, z, vx, vy, vz, r;
};

smk_sim* g_sim = nullptr;
std::vector<RefObject> g_objects;
float g_gravity = -9.82f;
float g_buoyancy = 2.0f;

void die(const char* what, int rc) {
    fprintf(stderr, "%s: %s (%s)\n", what, smk_error_string(rc), smk_last_error());
    exit(-1);
}

}  // namespace

void getGPUProperties(void) {
    int devices = 0;
    cudaError_t err = cudaGetDeviceCount(&devices);
    if (err != cudaSuccess) {
        fprintf(stderr, "Error finding available GPUs, now exiting\n");
        exit(-1);
    }
    for (int i = 0; i < devices; ++i) {
        cudaDeviceProp prop;
        printf("CUDA Device - ID %d\n", i);
        if (cudaGetDeviceProperties(&prop, i) == cudaSuccess) {
            printf("Max threads per block: \t\t%d\n", prop.maxThreadsPerBlock);
            printf("Max block dimensions: \t\t(%d, %d, %d)\n", prop.maxThreadsDim[0], prop.maxThreadsDim[1],
                   prop.maxThreadsDim[2]);
            printf("Max grid dimensions: \t\t(%d, %d, %d)\n", prop.maxGridSize[0], prop.maxGridSize[1],
                   prop.maxGridSize[2]);
            printf("Shared memory per block: \t%.2lfKB\n", prop.sharedMemPerBlock / 1024.);
        }
        printf("\n");
    }
}

void initializeVolume(float* smoke_grid, unsigned int width, unsigned int heigth, unsigned int depth) {
    if (g_sim) {
        smk_destroy(g_sim);
        g_sim = nullptr;
    }
    smk_params p;
    smk_default_params(&p);
    int rc = smk_create((int)width, (int)heigth, (int)depth, &p, &g_sim);
    if (rc) die("Error allocating smoke grid on GPU", rc);
    rc = smk_set_density(g_sim, smoke_grid);
    if (rc) die("Error copying data from host to device", rc);
}

void deleteVolume() {
    if (g_sim) smk_destroy(g_sim);
    g_sim = nullptr;
}

int addObstacle(float x, float y, float z, float vx, float vy, float vz, float r) {
    g_objects.push_back(RefObject{0, x, y, z, vx, vy, vz, r});
    return (int)g_objects.size() - 1;
}

int addSmokeSource(float x, float y, float z, float r) {
    g_objects.push_back(RefObject{1, x, y, z, 0.0f, 0.0f, 0.0f, r});
    return (int)g_objects.size() - 1;
}

void updateObjectPos(int id, float x, float y, float z) {
    if (id < 0 || id >= (int)g_objects.size()) {
        fprintf(stderr, "updateObjectPos: no object with id %d\n", id);
        return;
    }
    g_objects[id].x = x;
    g_objects[id].y = y;
    g_objects[id].z = z;
}

float* getBuoyancy() { return &g_buoyancy; }
float* getGravity() { return &g_gravity; }

void simulate(float* smoke_grid, float dt) {
    if (!g_sim) {
        fprintf(stderr, "simulate called before initializeVolume\n");
        exit(-1);
    }
    smk_params p;
    smk_get_params(g_sim, &p);
    p.gravity = g_gravity;
    p.buoyancy = g_buoyancy;
    int rc = smk_set_params(g_sim, &p);
    if (rc) die("Error setting parameters", rc);
    smk_clear_objects(g_sim);
    for (const RefObject& o : g_objects) {
        rc = o.type == 0 ? smk_add_obstacle(g_sim, o.x, o.y, o.z, o.vx, o.vy, o.vz, o.r, nullptr)
                         : smk_add_smoke_source(g_sim, o.x, o.y, o.z, o.r, nullptr);
        if (rc) die("Error registering objects", rc);
    }
    rc = smk_simulate(g_sim, smoke_grid, dt);
    if (rc) die("Error copying data from device to host", rc);
}
