"""Learned initial density for the SCF (6-31G, H/C/N/O): an atom-pair network
(blocks.py, mlp.py) trained on converged densities from this package's own batched
SCF (train.py).  The SAD guess stays the fallback and the SCF decides the result: the learned
density only seeds the iterations."""
