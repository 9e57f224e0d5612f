"""gbfe -- GB300-native FE operator apply / ChFSI / Poisson-CG hot path of dft-efe.

``gbfe.mesh`` generates inputs (numpy, host).  ``gbfe.api`` is the host mirror of
the reference's operator and solver interface; every compute call goes to the
CUDA library ``libgbfe.so`` (see include/gbfe.h).  Importing ``gbfe.api`` loads
that library and fails if it has not been built.
"""
from .build import build  # noqa: F401

__all__ = ["build"]
