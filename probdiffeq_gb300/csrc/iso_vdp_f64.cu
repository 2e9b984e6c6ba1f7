// Isotropic adaptive kernels for the VanDerPol field in double bulk precision.
#include "iso_launch.cuh"

PDQ_DEFINE_ISO_LAUNCH(pdq_launch_iso_vdp_f64, double, pdq::VanDerPol)
