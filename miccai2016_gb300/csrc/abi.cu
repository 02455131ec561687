// abi.cu -- status strings and the ABI version of the C interface.
#include "common.cuh"

extern "C" const char *m16_status_string(int status)
{
    switch (status) {
    case M16_OK: return "ok";
    case M16_ERR_BAD_SHAPE: return "bad shape";
    case M16_ERR_BAD_ARG: return "bad argument";
    case M16_ERR_WORKSPACE: return "workspace missing, misaligned or too small";
    case M16_ERR_CUDA: return "CUDA runtime error";
    case M16_ERR_TIMEOUT: return "device-side wait timed out";
    case M16_ERR_TOO_LARGE: return "request exceeds a fixed capacity (the no-allocation entry point's scratch or a server's work table)";
    default: return "unknown status";
    }
}

extern "C" int m16_abi_version(void) { return 5; }
