"""CPU oracle of the render-and-fit path: test infrastructure, never product code.

A float64 PyTorch (CPU) restatement of the reference's closed forms, used only by
tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the checker. The
product path (dirichlet-splatting_gb300/dsplat) never imports it.

Pinned: tests/test_oracle_golden.py checks these functions against golden vectors
that tests/golden/make_golden.py produced by running the reference's own float64
oracles (tests/reference/kernel.py, tests/reference/oracle.py and
dsplat/groundtruth.py of Asixa/Dirichlet-Splatting) on seeded inputs.

kernel    Dirichlet kernel and windows (tests/reference/kernel.py:8-57)
fmcw      surfel columns, analytic derivatives, render / JVP / VJP / correlations,
          ADC synthesis (dsplat/groundtruth.py:40-90, tests/reference/oracle.py:34-41,
          dsplat/kernels/scattering.slang:16-50)
adjoint   the reference VJP kernel's hand-derived adjoint (per-class cotangent sums, nearest
          bin apart, chain rule; dsplat/kernels/surfel.slang:227-311) in float64, pinned to
          autograd of the closed form by tests/test_oracle_adjoint.py
spectral  separable atoms and derivatives (tests/reference/oracle.py:10-31)
search    range gate, greedy peaks, quasi-Newton direction and trial step
          (dsplat/kernels/search.slang:7-109)
scene     the 13-DOF range/Doppler/azimuth renderer (dsplat/surfel.py:132-196,
          tests/reference/physics.py:11-25)
solver    the float64 VarPro refit timed as the CPU baseline (dsplat/varpro.py)
"""
