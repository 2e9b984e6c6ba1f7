// Split isotropic filter (covariance warp + mean warp) for the FitzHughNagumo field in double bulk precision.
#include "iso_split_launch.cuh"

PDQ_DEFINE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_fhn_f64, double, pdq::FitzHughNagumo)
