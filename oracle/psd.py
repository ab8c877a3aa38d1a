"""Batched PSD projection by eigenvalue flooring, FP64 restatement.

Reference: ``simkit/psd_project.py:12-47``.  Each symmetric block is
eigen-decomposed with LAPACK ``syevd`` (numpy ``eigh``); with
``method='proj'`` eigenvalues below 1e-6 are raised to 1e-6 (:37), with
``'abs'`` they are replaced by their magnitudes (:35); the block is rebuilt
as ``U diag(s) U^T`` (:46).
"""

from __future__ import annotations

import numpy as np

PSD_FLOOR = 1e-6


def psd_project(H, method: str = "proj") -> np.ndarray:
    H = np.asarray(H, dtype=np.float64)
    if H.ndim == 2:
        H = H[None]
    s, U = np.linalg.eigh(H)
    if method == "abs":
        s = np.abs(s)
    elif method == "proj":
        s = np.maximum(s, PSD_FLOOR)
    return np.einsum("tij,tj,tkj->tik", U, s, U)
