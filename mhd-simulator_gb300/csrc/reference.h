// reference.h -- the reference solver (FP32 Jacobi-CG / aggregation-MG CG with
// the reference's gauges and convergence tests) behind the same context.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "../../include/mhdproj.h"

namespace mhdproj {
struct RefState;
int ref_create(RefState** out, const mhdproj_grid* grid, const mhdproj_options* opt, cudaStream_t stream,
               std::string& err);
void ref_destroy(RefState* s);
void ref_set_stream(RefState* s, cudaStream_t stream);
int ref_set_topology(RefState* s, const uint32_t* mask_host, uint32_t components, std::string& err);
// The encoded mask in device memory (written by the GPU labelling), and the
// counts that go with it.
uint32_t* ref_mask(RefState* s);
void ref_set_topology_device(RefState* s, uint32_t components, uint32_t fluid_cells);
// What the fluid step and fields kernels read of the reference solver.
struct RefExport {
    const uint32_t* mask;
    const float* occ;
    const float* phase;  // null without phase drag
    const float* work;   // float4 per cell, x = pressure potential
    uint32_t fluid_cells;
    int mean_free, two_phase;
    float rho_l, rho_air, drag_rate, drag_dt;
};
RefExport ref_export(RefState* s);
int ref_set_coefficients(RefState* s, const float* alpha, float rho_l, float rho_air, std::string& err);
int ref_set_phase_drag(RefState* s, const float* phase, float drag_rate, float dt, std::string& err);
int ref_project(RefState* s, const float* us, const float* vs, const float* ws, float* uo, float* vo, float* wo,
                float* po, float dt, int warm, mhdproj_stats* st, std::string& err);
int ref_apply_operator(RefState* s, const float* x, float* y, std::string& err);
int ref_apply_preconditioner(RefState* s, const float* r, float* z, std::string& err);
int ref_copy_coefficients(RefState* s, float* coef4, std::string& err);
int ref_copy_potential(RefState* s, double* phi, std::string& err);
}  // namespace mhdproj
