// Isotropic adaptive kernels with the fixed-point smoother for the LotkaVolterra field in float bulk precision.
#include "iso_launch.cuh"

PDQ_DEFINE_ISO_FP_LAUNCH(pdq_launch_iso_fp_lv_f32, float, pdq::LotkaVolterra)
