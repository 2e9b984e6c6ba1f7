// Structure-exploiting dense kernel with eight or sixteen lanes per instance for the LotkaVolterra field in float
// bulk precision.
#include "dense_launch.cuh"

PDQ_DEFINE_DENSE_LANES_LAUNCH(pdq_launch_dense_lanes_lv_f32, float, pdq::LotkaVolterra)
