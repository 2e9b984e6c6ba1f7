// Split isotropic filter (covariance warp + mean warp) for the LotkaVolterra field in float bulk precision.
#include "iso_split_launch.cuh"

PDQ_DEFINE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_lv_f32, float, pdq::LotkaVolterra)
