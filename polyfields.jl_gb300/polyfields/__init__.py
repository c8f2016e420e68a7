"""polyfields — GB300 engine for PolyFields.jl's SCFT hot path, driven from Python.

The compute path is libpolyfields_gpu.so (hand-written sm_103a CUDA kernels behind the C ABI
of include/polyfields_gpu.h); this package mirrors the reference's public API on top of it.
"""
from .api import (AndersonUpdater, Canonical, Diblock, DomainUpdater, EdwardsInteraction, EulerUpdater, FieldSystem, FloryInteraction, FP32, FP64,
                  Grand, Homopolymer, MomentumUpdater, Monomer, Multiblock, Point, SCFTOptions, SCFTResults, UnitCell, add_cell,
                  add_interaction, add_monomer, add_species, chain_grid, monomer_fraction, uniform_fields, density, field_error, fieldinit, free_energy, free_energy_bulk, interpolate_grid,
                  loadfields,
                  residuals, savefields, scfstress, scft, scft_batch, set_interaction, setup, step,
                  updater_with_system, validate)
from ._lib import LIB_PATH, PolyFieldsError, load as load_library

__all__ = [n for n in dir() if not n.startswith("_")]
