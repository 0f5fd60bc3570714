"""fast_gb300 -- GB300-native tortuosity engine (the `fast tau` /
fastlib getTortuosity path of krsvojte/fast), served by libfasttau.so."""
from .tau import (DSOLVER_BICGSTAB, DSOLVER_CG, DiffusionSolverType, Dir, FaceMean, Precision, Status,
                  TauResult, TortuosityParams, Volume, get_porosity, get_tortuosity, solve_batch,
                  solve_batch_device, solve_directions, solve_directions_device)

__all__ = ["DSOLVER_BICGSTAB", "DSOLVER_CG", "DiffusionSolverType", "Dir", "FaceMean", "Precision", "Status",
           "TauResult", "TortuosityParams", "Volume", "get_porosity", "get_tortuosity", "solve_batch",
           "solve_batch_device", "solve_directions", "solve_directions_device"]
