/* Force-included into every reference translation unit of the oracle build.
 * The reference seeds its samplers with std::random_device (rchol_lap.cpp:685,
 * util.hpp:51), so no two runs agree.  This header declares a drop-in device
 * that returns a caller-chosen seed and renames random_device to it after
 * <random> has been parsed, which makes the unmodified reference
 * reproducible.  Test infrastructure only. */
#pragma once
#include <random>
extern "C" unsigned int oracle_ref_seed;
namespace std {
struct oracle_fixed_seed_device {
  typedef unsigned int result_type;
  result_type operator()() { return oracle_ref_seed; }
};
}  // namespace std
#define random_device oracle_fixed_seed_device
