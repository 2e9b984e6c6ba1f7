// Split isotropic filter (covariance warp + mean warp) for the VanDerPol field in double bulk precision.
#include "iso_split_launch.cuh"

PDQ_DEFINE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_vdp_f64, double, pdq::VanDerPol)
