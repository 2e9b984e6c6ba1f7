// Isotropic adaptive kernels for the VanDerPol field in float bulk precision.
#include "iso_launch.cuh"

PDQ_DEFINE_ISO_LAUNCH(pdq_launch_iso_vdp_f32, float, pdq::VanDerPol)
