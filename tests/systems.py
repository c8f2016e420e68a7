"""Test-side alias of the workload builders (polyfields.workloads)."""
from polyfields.workloads import (GOLDEN, blend3d_system, blend_seed_system, cyl2d_seed_system,  # noqa: F401
                                  diblock_system, seeded_fields)
