// seeded_random_device.h — forced into the reference's GaussianGeometry.cpp
// by oracle/build_ref.py (g++ -include), so that the std::random_device{}()
// that seeds GaussianPoint::random (GaussianGeometry.cpp:17) returns a seed
// the checker chooses (ref_random_points in ref_glue.cpp). <random> is
// included first, so the macro renames only the reference's own use.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <random>

namespace std {
struct tpd_seeded_random_device {
    unsigned int operator()() const;
};
}  // namespace std

#define random_device tpd_seeded_random_device
