"""Generate tests/golden/reference_periodic.npz from the reference's own code (CPU only).

Runs the reference's diffusion_2D sources, compiled unmodified into oracle/_ref by
``make -C oracle ref`` (single-rank MPI and serial N_Vector stand-ins), on the reference's
periodic problem (default domain [-pi, pi] x [-6, 6], dx = (xu-xl)/(nx-1)):

  ic            Initial (initial.cpp:20-47)
  f_hom, f_inh  the ARKRhsFn diffusion (diffusion.cpp:9-209) of a seeded random field u,
                homogeneous and inhomogeneous (k (1 + 0.99 sin), diffusion_2D.cpp:887-897)
                coefficients, at t = 0.3
  z_hom         PSetup + PSolve (preconditioner_jacobi.cpp:9-61) of r = u, gamma = 1e-3
  d_inh         the inhomogeneous PSetup diagonal (coefficients at nodes, :23-37)

The GPU tests compare the product's periodic RHS, initial state and Jacobi PSolve with these
outputs of the reference itself (the reference tree is not present beside the GPU).

Usage (from the repository root, where the reference tree is present):
    python tests/golden/make_reference_goldens.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import refbind as rb  # noqa: E402

NX, NY, KX, KY, T, GAMMA, SEED = 48, 40, 1.0, 0.5, 0.3, 1e-3, 20261204


def main():
    u = np.random.default_rng(SEED).standard_normal(NX * NY)
    H = rb.RefProblem(NX, NY, KX, KY, False)
    I = rb.RefProblem(NX, NY, KX, KY, True)
    d_hom, z_hom = H.jacobi(GAMMA, u)
    d_inh, _ = I.jacobi(GAMMA, u)
    np.savez_compressed(os.path.join(HERE, "reference_periodic.npz"), nx=NX, ny=NY, kx=KX, ky=KY, t=T,
                        gamma=GAMMA, seed=SEED, u=u, ic=H.initial(), f_hom=H.rhs(T, u), f_inh=I.rhs(T, u),
                        z_hom=z_hom, d_inh=d_inh)
    print("wrote reference_periodic.npz")


if __name__ == "__main__":
    main()
