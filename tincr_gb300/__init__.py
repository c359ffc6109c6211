"""tincr_gb300 — GB300 (sm_103a) implementation of tincr's linear-response excited-state path.

The compute path is the CUDA library built in-tree from `csrc/` (see build.py) and reached through
the C ABI of include/tincr_gb300.h; `tda.py` mirrors tincr's Rust interface on top of it.
`groundstate.py` is the host-side upstream producer of the path's inputs (C, S, orbital energies,
gamma matrices), not part of the GPU path.
"""

__all__ = ["build", "tda", "groundstate", "params"]
