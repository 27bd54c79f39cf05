"""Dense Hermitian solves of the solver and its preconditioned conjugate gradients.

Every system here is small (K x K with K the support size, at most a few thousand) and
lives on the GPU; cuSOLVER (through torch.linalg) factors it. The numerically delicate
part is the rank-deficient Gram of a support with a surfel no aperture sees, or two atoms
at one position: its Cholesky factor does not exist, and the solve instead factors
h + shift I in float64 with shift = (size * eps) * lambda_max(h), the level at which a
pseudoinverse would truncate. The shift only moves the solution along near-null
directions, which the prediction does not see. Semantics of the reference's
dsplat/varpro.py:29-79 (power iteration start, shift schedule) and varpro.py:206-228 (PCG).

GB300 choices: each data-dependent decision reads one small device tensor (a factor's
status with its diagnostics); a float64 system that must be shifted is first solved from a
float32 factor with float64 refinement (a float32 Cholesky of 2000^2 costs a seventh of the
float64 one here); and PCG runs a fixed number of iterations with its stopping rule kept
as a device-side flag, looking at it only every few iterations.
"""

from __future__ import annotations

import torch

from .graphs import recording, side_stream

POWER_STEPS = 24  # power iterations for the largest eigenvalue of a Gram
SHIFT_RETRIES = 4
# Cumulative shift multipliers of the retries: each retry adds nine times everything
# added so far (1, 1 + 9, 10 + 81, 91 + 729).
SHIFT_LADDER = (1, 10, 91, 820)[:SHIFT_RETRIES]
PCG_CHECK_EVERY = 4  # iterations between host reads of the PCG stopping flag


def _wide(h):
    """h in float64 (complex128 when complex), as a fresh tensor."""
    return h.to(torch.complex128 if h.is_complex() else torch.float64, copy=True)


def largest_eigenvalue(h):
    """Power-iteration estimate of the largest eigenvalue of a positive semidefinite h.

    The start vector is the fixed golden-ratio sequence frac(0.618 i) + 0.5, so the
    estimate is reproducible without a generator.
    """
    ramp = torch.arange(len(h), device=h.device, dtype=torch.float64)
    v = (torch.remainder(ramp * 0.6180339887, 1) + 0.5).to(h.dtype)
    length = v.norm()
    for _ in range(POWER_STEPS):
        v = h @ v
        length = v.norm()
        v = v / length.clamp(min=torch.finfo(length.dtype).tiny)
    return length


def shifted_cholesky(h, floor):
    """Float64 Cholesky factor of h + shift I, or None when every retry fails.

    shift = floor * lambda_max(h) at first; after a failure the diagonal gets nine times
    the total shift so far, at most SHIFT_RETRIES attempts.
    """
    base = _wide(h)
    unit = floor * largest_eigenvalue(base)
    diagonal = base.diagonal().clone()
    for multiple in SHIFT_LADDER:
        base.diagonal().copy_(diagonal + multiple * unit)
        factor, status = torch.linalg.cholesky_ex(base)
        if int(status) == 0:
            return factor
    return None


class RefinedSolver:
    """Solves of a float64 h from one float32 Cholesky factor, with float64 refinement.

    The factor L is inverted once (X = L^-1, a triangular solve with the identity), so each
    correction is two matrix-vector products X^H (X r) instead of two sequential triangular
    solves; the float64 refinement then converges exactly as with the factor (each step
    shrinks the error by about cond(h) float32 epsilon either way). Factoring once also lets
    a refinement loop over several right-hand sides reuse it.
    """

    def __init__(self, h):
        low = torch.complex64 if h.is_complex() else torch.float32
        factor, self.status = torch.linalg.cholesky_ex(h.to(low))
        eye = torch.eye(len(h), dtype=low, device=h.device)
        self.inverse_factor = torch.linalg.solve_triangular(factor, eye, upper=False)
        self.h = h
        self.norm = torch.linalg.matrix_norm(h)

    def _apply(self, r):
        x = self.inverse_factor
        return (x.mH @ (x @ r.to(x.dtype))).to(self.h.dtype)

    def __call__(self, rhs, iterations=3, tolerance=1e-13):
        """x = h^-1 rhs, or None when the factor does not exist or the normwise backward
        error |q - h x| / (|h|_F |x| + |q|) stays above tolerance (one device read)."""
        q = (rhs if rhs.ndim == 2 else rhs[:, None]).to(self.h.dtype)
        x = self._apply(q)
        for _ in range(iterations):
            x = x + self._apply(q - self.h @ x)
        scale = self.norm * x.norm() + q.norm()
        error = (q - self.h @ x).norm() / scale.clamp(min=1e-300)
        verdict = (self.status == 0) & (error <= tolerance)  # a failed factor leaves NaN in error
        if not bool(verdict):
            return None
        return x if rhs.ndim == 2 else x[:, 0]


def refined_solve(h, rhs, iterations=3, tolerance=1e-13):
    """x = h^-1 rhs for a float64 h from a float32 factor with float64 iterative refinement.

    Returns None, and the caller factors in float64, when the float32 factor does not
    exist or the normwise backward error |q - h x| / (|h|_F |x| + |q|) stays above
    tolerance (systems whose condition number nears 1 / float32 epsilon). One device read
    decides both.
    """
    return RefinedSolver(h)(rhs, iterations, tolerance)


def shifted_refined_solve(h, q, floor):
    """(h + floor lambda_max(h) I)^-1 q at the first shift of shifted_cholesky, or None."""
    base = _wide(h)
    base.diagonal().add_(floor * largest_eigenvalue(base))
    return refined_solve(base, q)


def factored_solver(h, refined=False):
    """solve(h, .) as a function of the right-hand side, with h factored once.

    The first call decides the factorization exactly as solve does (float32 / float64
    Cholesky, the shifted refined solve, or the shifted float64 factor); later calls reuse
    it, so a refinement loop costs one factorization.
    """
    floor = len(h) * torch.finfo(h.real.dtype).eps
    speculative = None
    if refined and h.is_cuda:
        # The shifted system's factor is needed exactly when h has no Cholesky factor, which
        # only the factorization below tells; both are latency bound, so the shifted one is
        # enqueued on the side stream first and runs beside it (wasted when h factors).
        current = torch.cuda.current_stream()
        side = side_stream(current.device, lane=1)
        side.wait_stream(current)
        with torch.cuda.stream(side):
            shifted = _wide(h)
            shifted.diagonal().add_(floor * largest_eigenvalue(shifted))
            speculative = RefinedSolver(shifted)
    factor, status = torch.linalg.cholesky_ex(h)
    failed = int(status) != 0
    if speculative is not None:
        current.wait_stream(side)
        for tensor in (speculative.h, speculative.inverse_factor, speculative.status, speculative.norm):
            tensor.record_stream(current)  # made on the side stream, used and freed on this one
    if not failed:
        return lambda rhs: _apply_factor(factor, rhs)
    if speculative is not None:
        solver = speculative  # factored once for every right-hand side

        def refined_call(rhs):
            q = rhs if rhs.ndim == 2 else rhs[:, None]
            x = solver(q)
            if x is None:
                return solve(h, rhs, refined=False)
            return (x if rhs.ndim == 2 else x[:, 0]).to(rhs.dtype)

        return refined_call
    wide_factor = shifted_cholesky(h, floor)
    if wide_factor is None:
        return torch.zeros_like
    return lambda rhs: _apply_factor(wide_factor, rhs)


def _apply_factor(factor, rhs):
    q = rhs if rhs.ndim == 2 else rhs[:, None]
    x = torch.cholesky_solve(q.to(factor.dtype), factor).to(q.dtype)
    return x if rhs.ndim == 2 else x[:, 0]


def solve(h, rhs, refined=False):
    """Hermitian solve; a singular h is shifted to where a pseudoinverse would truncate.

    refined first tries the shifted system through refined_solve (float32 factor, float64
    refinement), which gives its solution to float64 accuracy like the float64 factor.
    A Gram whose columns are all zero has nothing to fit: the answer is zero.
    """
    q = rhs if rhs.ndim == 2 else rhs[:, None]
    factor, status = torch.linalg.cholesky_ex(h)
    if int(status) != 0:
        floor = len(h) * torch.finfo(h.real.dtype).eps
        if refined and h.is_cuda:
            x = shifted_refined_solve(h, q, floor)
            if x is not None:
                return (x if rhs.ndim == 2 else x[:, 0]).to(rhs.dtype)
        factor = shifted_cholesky(h, floor)
        if factor is None:
            return torch.zeros_like(rhs)
    x = torch.cholesky_solve(q.to(factor.dtype), factor).to(q.dtype)
    return x if rhs.ndim == 2 else x[:, 0]


def pcg(operator, rhs, diagonal, *, iterations=32, tolerance=1e-3, capture=False):
    """Jacobi-preconditioned conjugate gradients from zero.

    Stops (keeps x) at the first direction of nonpositive curvature, or after the update
    that brings |r| to tolerance * |rhs| or below. The stop is a device flag: iterations
    after it change nothing. Eagerly the host looks at the flag every PCG_CHECK_EVERY
    iterations to skip the rest; with capture (CUDA tensors, and an operator that reads
    no device value) the first iteration runs eagerly and the others replay it from a
    CUDA graph, all iterations, with no device read at all.
    """
    if capture and rhs.is_cuda and iterations > 1:
        return _pcg_graphed(operator, rhs, diagonal, iterations, tolerance)
    x = torch.zeros_like(rhs)
    goal = tolerance * rhs.norm()
    r = rhs.clone()
    z = r / diagonal
    p = z.clone()
    rz = r @ z
    live = torch.ones((), dtype=torch.bool, device=rhs.device)
    for done in range(iterations):
        if done and done % PCG_CHECK_EVERY == 0 and not bool(live):
            break
        hp = operator(p)
        curvature = p @ hp
        live = live & (curvature > 0)
        alpha = rz / curvature
        x = torch.where(live, x + alpha * p, x)
        r = torch.where(live, r - alpha * hp, r)
        going = live & (r.norm() > goal)
        z = r / diagonal
        rz_next = r @ z
        p = torch.where(going, z + (rz_next / rz) * p, p)
        rz = torch.where(going, rz_next, rz)
        live = going
    return x


def _pcg_graphed(operator, rhs, diagonal, iterations, tolerance):
    """pcg with every iteration after the first replayed from one captured CUDA graph.

    The iterates live in static buffers that one iteration updates in place; the graph is
    captured per call (the operator's tensors belong to one Gauss-Newton system).
    """
    from .kernels import _lib

    goal = tolerance * rhs.norm()
    x = torch.zeros_like(rhs)
    r = rhs.clone()
    p = r / diagonal
    rz = (r @ p).reshape(())
    live = torch.ones((), dtype=torch.bool, device=rhs.device)

    def iteration():
        hp = operator(p)
        curvature = p @ hp
        moving = live & (curvature > 0)
        alpha = rz / curvature
        x.copy_(torch.where(moving, x + alpha * p, x))
        r_next = torch.where(moving, r - alpha * hp, r)
        going = moving & (r_next.norm() > goal)
        z = r_next / diagonal
        rz_next = r_next @ z
        p.copy_(torch.where(going, z + (rz_next / rz) * p, p))
        rz.copy_(torch.where(going, rz_next, rz))
        r.copy_(r_next)
        live.copy_(going)

    device = rhs.device
    side = side_stream(device)
    side.wait_stream(torch.cuda.current_stream(device))
    timers, _lib.TIMERS = _lib.TIMERS, None  # events cannot be recorded inside a capture
    try:
        with torch.cuda.stream(side):
            iteration()  # the first iteration, which is also the capture's warm-up
        torch.cuda.current_stream(device).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        before = _lib.library().dsg_launch_count()
        with recording(graph):
            iteration()
        per_replay = _lib.library().dsg_launch_count() - before
        for _ in range(iterations - 1):
            graph.replay()
        _lib.REPLAYED_LAUNCHES += per_replay * (iterations - 1)
    finally:
        _lib.TIMERS = timers
    return x.clone()


class GraphedPCG:
    """pcg's iterations replayed from one CUDA graph kept across solves of the same shapes.

    The operator must read only tensors whose addresses stay fixed (the caller refills
    them between solves); the iterates live in static buffers here. Construction runs one
    iteration eagerly (the capture's warm-up) and captures the next; every solve then
    reloads the start (x = 0, r = rhs, p = r / diagonal) and replays all iterations, with no
    device read. The arithmetic is that of pcg.
    """

    def __init__(self, operator, rhs, diagonal, iterations, tolerance):
        from .kernels import _lib

        self.iterations, self.tolerance = iterations, tolerance
        self.diagonal = diagonal.clone()
        self.x = torch.zeros_like(rhs)
        self.r = rhs.clone()
        self.p = torch.zeros_like(rhs)
        self.rz = rhs.new_zeros(())
        self.goal = rhs.new_zeros(())
        self.live = torch.ones((), dtype=torch.bool, device=rhs.device)
        x, r, p, rz, live, goal, diag = self.x, self.r, self.p, self.rz, self.live, self.goal, self.diagonal

        def iteration():
            hp = operator(p)
            curvature = p @ hp
            moving = live & (curvature > 0)
            alpha = rz / curvature
            x.copy_(torch.where(moving, x + alpha * p, x))
            r_next = torch.where(moving, r - alpha * hp, r)
            going = moving & (r_next.norm() > goal)
            z = r_next / diag
            rz_next = r_next @ z
            p.copy_(torch.where(going, z + (rz_next / rz) * p, p))
            rz.copy_(torch.where(going, rz_next, rz))
            r.copy_(r_next)
            live.copy_(going)

        device = rhs.device
        timers, _lib.TIMERS = _lib.TIMERS, None  # events cannot be recorded inside a capture
        try:
            self._load(rhs, diagonal)
            side = side_stream(device)
            side.wait_stream(torch.cuda.current_stream(device))
            with torch.cuda.stream(side):
                iteration()  # warm-up: lazy library set-up happens outside the capture
            torch.cuda.current_stream(device).wait_stream(side)
            self.graph = torch.cuda.CUDAGraph()
            before = _lib.library().dsg_launch_count()
            with recording(self.graph):
                iteration()
            self.per_replay = _lib.library().dsg_launch_count() - before
        finally:
            _lib.TIMERS = timers

    def _load(self, rhs, diagonal):
        self.diagonal.copy_(diagonal)
        self.x.zero_()
        self.r.copy_(rhs)
        torch.div(rhs, diagonal, out=self.p)
        self.rz.copy_(rhs @ self.p)
        self.goal.copy_(self.tolerance * rhs.norm())
        self.live.fill_(True)

    def solve(self, rhs, diagonal):
        """pcg(operator, rhs, diagonal) over the operator's current static inputs."""
        from .kernels import _lib

        self._load(rhs, diagonal)
        for _ in range(self.iterations):
            self.graph.replay()
        _lib.REPLAYED_LAUNCHES += self.per_replay * self.iterations
        return self.x.clone()
