// Terminal-value adjoint (record pass and adjoint pass) for the LotkaVolterra field in double bulk precision.
#include "tv_launch.cuh"

PDQ_DEFINE_TV_LAUNCH(pdq_launch_tv_lv_f64, double, pdq::LotkaVolterra)
