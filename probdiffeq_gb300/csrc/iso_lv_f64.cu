// Isotropic adaptive kernels for the LotkaVolterra field in double bulk precision.
#include "iso_launch.cuh"

PDQ_DEFINE_ISO_LAUNCH(pdq_launch_iso_lv_f64, double, pdq::LotkaVolterra)
