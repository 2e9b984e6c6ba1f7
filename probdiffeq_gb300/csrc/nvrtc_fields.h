// Internal interface between the C ABI dispatch and the run-time compiled
// user vector fields (nvrtc_fields.cu).
#pragma once

#include <cuda_runtime.h>

#include "bd_solver.cuh"
#include "dense_solver.cuh"
#include "iso_solver.cuh"
#include "lml_adjoint.cuh"

// State dimension / number of parameters of a registered user field (0 / -1 if unknown).
int pdq_user_field_dim(int32_t field);
int pdq_user_field_params(int32_t field);
// Whether a registered id is a block-diagonal stencil (pdq_register_stencil).
bool pdq_user_field_is_stencil(int32_t field);

// Launch the isotropic kernel instantiated for a registered user field;
// compiles and loads the variant on first use.
cudaError_t pdq_launch_iso_user(const pdq::IsoArgs& a, int32_t field, bool f64, int nu, bool interp, bool fp,
                                cudaStream_t stream, int block);

// The same for the dense kernel (one thread per instance).
cudaError_t pdq_launch_dense_user(const pdq::DenseArgs& a, int32_t field, bool f64, int nu, bool ts1, bool fp,
                                  cudaStream_t stream);

// The LML kernels for a registered user field: forward-mode gradient
// (pdq_lml_fixed_grid), and the adjoint pair's value / adjoint pass
// (pdq_lml_fwd / pdq_lml_bwd); the covariance plan kernel from the same module.
cudaError_t pdq_launch_lml_user(const pdq::LmlArgs& a, int32_t field, bool f64, int nu, cudaStream_t stream);
cudaError_t pdq_launch_lml_adj_user(const pdq::LmlAdjArgs& aa, int32_t field, bool f64, int nu, bool backward,
                                    cudaStream_t stream);

// The block-diagonal cluster kernel instantiated for a registered user
// stencil (struct Stencil); compiles and loads the variant on first use.
cudaError_t pdq_launch_bd_user(const pdq::BdArgs& a, int32_t field, bool f64, int nu, cudaStream_t stream);
