"""GB300-native RKHEVI dynamical-core step of GAME (MHBalsmeier/GAME_archived).

The product is the CUDA library libgame_gb300.so behind the C ABI in
include/game_gb300.h, which keeps the reference's own entry points
(manage_rkhevi, grad, divv_h, calc_pot_vort, vorticity_flux, ...).  This
package holds its sources (csrc/), the in-tree build, the grid-table builder
and the Python host-side mirror used by the tests and the benchmark.
"""
__all__ = ["abi", "build", "cases", "driver", "native", "ops", "structs", "tables"]
