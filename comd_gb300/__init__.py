"""comd_gb300: CoMD's force-and-integrate timestep on GB300 (sm_103a).

The product is ``libcomdgb.so`` (C ABI in ``include/comdgb.h``): link-cell
binning, LJ and EAM (table or Chebyshev) force kernels in FP64 or mixed
precision, and the velocity-Verlet loop, driven from C as a drop-in for the
reference's ``simflat_t`` / ``pot->force`` / ``nTimeSteps``.  This Python
package only builds and binds the library for tests and benchmarks.
"""
from . import abi
from .lib import (CLSMAN_BINARY, CLSMAN_TEXT, CLSMAN_TEXT_GZ, DATA_DIR, DISP_GAUSSIAN,
                  DISP_NONE, DISP_UNIFORM, ERR_BOXRANGE, ERR_MAXATOMS, ERR_NOBOX, POT_DIR,
                  POT_EAM_CHEBY, POT_EAM_TABLE, POT_LJ, PREC_FP64, PREC_MIXED, Batch,
                  ComdgbError, DeviceSim, Tune, batch_autotune, eam_potential, fcc, free_host,
                  lj_potential, load, opts, print_it, read_clsman, read_tim, rebin_host,
                  round_f32, seed, set_comment, write_clsman_host)

__all__ = ["abi", "load", "Batch", "opts", "DeviceSim", "ComdgbError", "eam_potential",
           "lj_potential", "fcc", "read_clsman", "read_tim", "write_clsman_host", "set_comment", "print_it",
           "DATA_DIR", "seed", "free_host", "round_f32", "POT_DIR", "POT_EAM_TABLE",
           "POT_EAM_CHEBY", "POT_LJ", "PREC_FP64", "PREC_MIXED", "DISP_NONE", "DISP_UNIFORM",
           "DISP_GAUSSIAN", "CLSMAN_BINARY", "CLSMAN_TEXT_GZ", "CLSMAN_TEXT", "ERR_MAXATOMS",
           "ERR_BOXRANGE", "ERR_NOBOX", "Tune", "batch_autotune", "rebin_host"]
