// io.cpp -- file-level module call (fpl_process), mirroring evd_process.
#include <cstring>

#include "fringe_gb300.h"

extern "C" {

void fpl_options_default(fpl_options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    // evdOptions::evdOptions, src/evd/evd.hpp:58-68
    o->blocksize = 64;
    o->memsize = 2048;
    o->Nx = 5;
    o->Ny = 5;
    o->minNeighbors = 2;
    o->miniStackCount = 1;
    o->method = "MLE";
    o->bandWidth = -1;
    o->semantics = FPL_SEM_EVD;
    o->precision = FPL_PREC_FP32;
    o->device = 0;
    o->verbose = 1;
}

int fpl_process(const fpl_options *opts)
{
    (void)opts;
    return FPL_ERR_UNSUPPORTED;
}

}
