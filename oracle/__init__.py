"""CPU oracle for the FAME bi-anisotropic eigensolver hot path.

TEST INFRASTRUCTURE ONLY.  This package is a literal FP64 restatement, in
NumPy/SciPy, of the reference MATLAB path (FAME-GPU/3D-Bi-Anisotropic-PhC):
the quasi-periodic curl-SVD data, the FFT transforms, the vertex-interpolated
material operators, the ``fncA``/``fncB``/``fncinvB`` handles, the Lanczos
band solver and the residual checks.  Every function cites the reference file
and line it follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference arms may import it, and only as the checker or the timed CPU
baseline.  The product library never routes through it.

Parity status: the reference ships no golden vectors and MATLAB is not
available, so this restatement is pinned by the reference's own in-code
identity checks (``Funhand_Generate_Lanzcos.m:176-219``,
``SVD_Matrix_Generate.m:59-102``, ``SVD_Matrix_1D.m:49-59``) evaluated against
the explicit sparse curl, and by closed-form eigenvalues of homogeneous media
(derived, not from the reference).
"""
from .fame_oracle import *  # noqa: F401,F403
