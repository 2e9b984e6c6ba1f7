// Dense-factorisation adaptive kernels for the LotkaVolterra field in double bulk precision.
#include "dense_launch.cuh"

PDQ_DEFINE_DENSE_LAUNCH(pdq_launch_dense_lv_f64, double, pdq::LotkaVolterra)
