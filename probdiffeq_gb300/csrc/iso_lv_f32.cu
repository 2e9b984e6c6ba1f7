// Isotropic adaptive kernels for the LotkaVolterra field in float bulk precision.
#include "iso_launch.cuh"

PDQ_DEFINE_ISO_LAUNCH(pdq_launch_iso_lv_f32, float, pdq::LotkaVolterra)
