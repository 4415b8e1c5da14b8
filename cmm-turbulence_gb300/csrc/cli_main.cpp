// cli_main.cpp -- SimulationCuda2d.out drop-in: `SimulationCuda2d.out
// [param_file=F] [COMMAND=VALUE ...]` (reference src/main2d.cpp:66-105),
// running the GB300 library through its C-ABI.
#include <cstdio>

#include "../../include/cmm_abi.h"

int main(int argc, char** argv)
{
    cmm_ctx* ctx = nullptr;
    int rc = cmm_create(argc, argv, &ctx);
    if (rc != CMM_OK) {
        fprintf(stderr, "cmm: %s\n", cmm_last_error());
        return 1;
    }
    rc = cmm_init(ctx);
    if (rc == CMM_OK || rc == CMM_ERR_SATURATED) rc = cmm_run(ctx);
    if (rc != CMM_OK && rc != CMM_ERR_SATURATED) fprintf(stderr, "cmm: %s\n", cmm_last_error());
    cmm_destroy(ctx);
    return (rc == CMM_OK || rc == CMM_ERR_SATURATED) ? 0 : 1;
}
