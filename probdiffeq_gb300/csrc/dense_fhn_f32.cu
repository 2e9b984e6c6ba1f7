// Dense-factorisation adaptive kernels for the FitzHughNagumo field in float bulk precision.
#include "dense_launch.cuh"

PDQ_DEFINE_DENSE_LAUNCH(pdq_launch_dense_fhn_f32, float, pdq::FitzHughNagumo)
