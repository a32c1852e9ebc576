"""GB300-native lattice-Boltzmann step for SFCMM/LBM.

Modules (each loads the CUDA library on first use; there is no CPU fallback):

* ``solver``: ``LBMSolver`` (the reference's run loop), ``TableSolver``
  (reference-table engine), ``BoxSolver`` (dense-box engine), ``BatchSolver``
  (batched cavities);
* ``refconfig``: the reference's JSON ``solver`` block to constants and
  boundary objects;
* ``gridgen``: the reference's grid and tables from a JSON config (host or GPU);
* ``lpt``: Lagrangian particles (``ParticleSolver``);
* ``output``: the reference's VTK PolyData file and ``line.csv`` probes;
* ``warmstart``: the learned warm start (U-Net);
* ``cases``: the benchmark configurations.
"""
