// Terminal-value adjoint (record pass and adjoint pass) for the VanDerPol field in float bulk precision.
#include "tv_launch.cuh"

PDQ_DEFINE_TV_LAUNCH(pdq_launch_tv_vdp_f32, float, pdq::VanDerPol)
