"""porescale_gb300 -- GB300 (sm_103a) implementation of porescale's hot paths.

Python side of the C ABI declared in ``include/porescale.h``:

* :class:`Lattice` -- the D3Q19 colour-gradient two-phase lattice (the
  reference's ``majorityrule`` step, S1:3634-3945 of
  LBM-LSM/lsm_lbm_static_alpha_beta_multipore.f);
* :class:`LatticeBatch` -- many such lattices advanced by shared
  persistent launches replayed from a CUDA graph;
* :class:`SpringNetwork` -- the alpha-beta / bond-bending lattice-spring
  static solve (LSM2S/Cxxxx/XX_P.f, LSM2S/Cyzyz/YZ_P.f).

The shared library ``libporescale_gpu.so`` is built in-tree by
``__graft_entry__.build()`` (or ``python porescale_gb300/_build.py``).  There
is no CPU fallback: if the library is missing, importing the bindings raises.
"""
from __future__ import annotations

from ._lib import (PREC_BF16, PREC_F16, PREC_F32, PREC_F64, PREC_NAMES, LbmInfo, LbmObs, LbmParams, PorescaleError,
                   library, library_path)
from .lattice import Lattice, LatticeBatch
from .springs import SpringNetwork, spring_constants

__all__ = [
    "Lattice", "LatticeBatch", "SpringNetwork", "spring_constants", "LbmParams", "LbmInfo", "LbmObs", "PorescaleError", "library", "library_path",
    "PREC_F64", "PREC_F32", "PREC_F16", "PREC_BF16", "PREC_NAMES",
]
