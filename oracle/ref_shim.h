// Force-included ahead of the reference headers by oracle/build.py (test infrastructure).
// The reference seeds mt19937 from std::random_device (kshape.cuh:163-164), which
// cannot be reproduced.  This shim replaces that one name with a device that returns
// a seed chosen by the harness, so the reference's own randomSelectK can be run with
// a known seed.  No reference source is edited.
#ifndef TC_REF_SHIM_H
#define TC_REF_SHIM_H
#include <random>
extern unsigned int tc_ref_seed;
struct tc_seeded_device {
    typedef unsigned int result_type;
    unsigned int operator()() { return tc_ref_seed; }
};
#define random_device tc_seeded_device
#endif
