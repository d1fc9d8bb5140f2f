"""swalbe_gb300 -- GB300-native thin-film lattice Boltzmann time step.

A drop-in for the time loop of Swalbe.jl: the same API (SysConst, Taumucs,
Sys, time_loop, run_*) over a CUDA C-ABI library for sm_103a.
"""
from .api import (Batch, BGKandStream_, GB300State, Server, Sys, SysConst, Taumucs, cospi,
                  count_droplets, boxpattern, ellipsepattern, trianglepattern, snapshot_,
                  save_snapshots, restart_from_height,
                  equilibrium_, filmpressure_, force_sum_, h_grad_p_, inclination_, moments_,
                  randinterface_, run_dropletforced, run_dropletpatterned, run_dropletrelax,
                  run_flat, run_random, run_rayleightaylor, singledroplet, slippage_,
                  surfacearea_, time_loop, two_caps, wetted_, launch_count)
from ._lib import SwbError, lib
from .d1 import Batch1D, State1D, SysConst_1D, run_gamma, two_droplets
from .build import LIB_PATH, build

__all__ = [
    "Batch", "BGKandStream_", "GB300State", "Server", "Sys", "SysConst", "Taumucs", "cospi",
    "Batch1D", "State1D", "SysConst_1D", "run_gamma", "two_droplets", "count_droplets", "boxpattern", "ellipsepattern", "trianglepattern", "snapshot_",
    "save_snapshots", "restart_from_height",
    "equilibrium_", "filmpressure_", "force_sum_", "h_grad_p_", "inclination_", "moments_",
    "randinterface_", "run_dropletforced", "run_dropletpatterned", "run_dropletrelax", "run_flat",
    "run_random", "run_rayleightaylor", "singledroplet", "slippage_", "surfacearea_", "time_loop",
    "two_caps", "wetted_", "launch_count", "SwbError", "lib", "LIB_PATH", "build",
]
