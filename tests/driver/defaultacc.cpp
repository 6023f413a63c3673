// Build-time setting for the driver linked against libhzgb300.so (test
// infrastructure): the reference objects it is compared with were compiled
// with -DDEFAULTACC=1e-13; the library's counterpart of that compile-time
// switch is hz_ref_config.bicg_acc, set here before main() runs.
#include "helmholtz_ref_api.h"

namespace {
struct SetDefaultAcc {
    SetDefaultAcc()
    {
        hz_ref_config c;
        hz_ref_get_config(&c);
        c.bicg_acc = 1e-13;
        hz_ref_set_config(&c);
    }
} set_default_acc;
}  // namespace
