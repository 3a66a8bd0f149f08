// smokeSimulation_gb300.cuh -- the reference's simulation interface, exported unchanged by
// libsmoke_gb300 so that its callers (project/main.cpp, project/boundingBox.cpp) link against
// this library without source changes.
//
// Each declaration replaces the function of the same signature in the reference's
// project/smokeSimulation.cuh (lines cited).  C++ linkage, one implicit simulation, CUDA and
// argument errors print to stderr and exit(-1) as the reference does.  The handle-based C ABI
// with status codes is include/smoke_gb300.h.
#pragma once
#include <vector>

void getGPUProperties(void);                                        // smokeSimulation.cuh:4
void simulate(float* smoke_grid, float dt);                         // smokeSimulation.cuh:6
void initializeVolume(float* smoke_grid, unsigned int width,        // smokeSimulation.cuh:8
                      unsigned int heigth, unsigned int depth);
void deleteVolume();                                                // smokeSimulation.cuh:9
int addObstacle(float x, float y, float z, float vx, float vy,      // smokeSimulation.cuh:12
                float vz, float r);
int addSmokeSource(float x, float y, float z, float r);             // smokeSimulation.cuh:13
void updateObjectPos(int id, float x, float y, float z);            // smokeSimulation.cuh:14
float* getBuoyancy();                                               // smokeSimulation.cuh:16
float* getGravity();                                                // smokeSimulation.cuh:17
