// Override of the reference's define_float_type.h that selects double scalars (the
// reference ships float; its commented-out lines pick the double aliases).  Used only
// by oracle/build_ref.sh for the double build of the reference translation units.
#pragma once
#include <Eigen/Dense>
using MY_FLOAT_TYPE = double;
using VEC2_TYPE = Eigen::Vector2d;
using VEC3_TYPE = Eigen::Vector3d;
using MAT3_TYPE = Eigen::Matrix3d;
