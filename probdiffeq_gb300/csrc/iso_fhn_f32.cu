// Isotropic adaptive kernels for the FitzHughNagumo field in float bulk precision.
#include "iso_launch.cuh"

PDQ_DEFINE_ISO_LAUNCH(pdq_launch_iso_fhn_f32, float, pdq::FitzHughNagumo)
