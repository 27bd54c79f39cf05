"""Oriented surfels, the scattering primitive of the FMCW measurements.

A surfel has a center [3] (m), an outward unit normal [3] and an area (m^2); its
reflectivity b is the linear coefficient variable projection solves, its material a
known refractive index fresnel_n (<= 1 for none). Seen from a monostatic sensor at
p, with r = |p - c|, u = (p - c) / r and cos = u . n:

    amplitude = sqrt(area) cos^2 F(cos) lambda / (8 pi r)     zero when cos <= 0
    F(cos)    = (root - cos) / (root + cos),  root = sqrt(fresnel_n^2 - 1 + cos^2)
    delay     = 2 r / c

The echo depends on area and reflectivity only through w = b sqrt(area). These
functions carry that area chain around the CUDA kernels of dsplat.kernels.surfel
(reference: dsplat/surfel.py:45-129).
"""

from __future__ import annotations

from .kernels import surfel as kernel


def render(config, positions, params, coefficients, fresnel_n=0.0):
    """Range profiles [A, K] of surfels with reflectivities coefficients; differentiable."""
    weights = coefficients * params["areas"].sqrt()
    return kernel.render(config, positions, params["centers"], params["normals"], weights, fresnel_n)


def jvp(config, positions, params, coefficients, tangent, delta_coefficients, fresnel_n=0.0):
    """Change of the profiles along tangent (centers, normals, areas) and delta_coefficients.

    With s = sqrt(area): dw = db s + b d(area) / (2 s).
    """
    root = params["areas"].sqrt()
    weights = coefficients * root
    delta_weights = delta_coefficients * root + coefficients * tangent["areas"] / (2 * root)
    return kernel.jvp(
        config, positions, params["centers"], params["normals"], weights,
        tangent["centers"], tangent["normals"], delta_weights, fresnel_n,
    )  # fmt: skip


def vjp(config, positions, params, coefficients, upstream, fresnel_n=0.0):
    """Gradients of Re(conj(upstream) . profiles) per parameter and for the coefficients."""
    root = params["areas"].sqrt()
    centers, normals, grad_weights = kernel.vjp(
        config, positions, params["centers"], params["normals"], coefficients * root, upstream,
        fresnel_n,
    )  # fmt: skip
    areas = (grad_weights.conj() * coefficients).real / (2 * root)
    return dict(centers=centers, normals=normals, areas=areas), grad_weights * root


def design(config, positions, params, fresnel_n=0.0, real=False):
    """Dictionary columns of every surfel for whole apertures; see kernels.surfel.design."""
    return kernel.design(
        config, positions, params["centers"], params["normals"], params["areas"], fresnel_n, real
    )


def jacobian(config, positions, params, fresnel_n=0.0):
    """Derivatives of the columns [A, K, S] by centers and normals [..., 3] and areas [..., 1]."""
    columns, dc, dn = kernel.jacobian(config, positions, params["centers"], params["normals"], fresnel_n)
    root = params["areas"].sqrt()
    return {
        "centers": dc * root[:, None],
        "normals": dn * root[:, None],
        "areas": (columns / (2 * root))[..., None],
    }


def correlate(config, positions, params, residual, fresnel_n=0.0, active=None):
    """a^H r and |a|^2 of every surfel's column a against the residual profiles [A, K].

    active (count tensor, period) restricts the work to surfels whose index mod period is
    below count (the others return zeros).
    """
    corr, norm = kernel.correlate(
        config, positions, params["centers"], params["normals"], residual, fresnel_n, active
    )
    return corr * params["areas"].sqrt(), norm * params["areas"]


def correlate_gradient(config, positions, params, residual, fresnel_n=0.0, include_normals=False):
    """correlate and its derivatives by centers (and normals): corr, norm, dcorr, dnorm."""
    corr, norm, dcorr, dnorm = kernel.correlate_gradient(
        config, positions, params["centers"], params["normals"], residual, fresnel_n,
        include_normals,
    )  # fmt: skip
    root, area = params["areas"].sqrt(), params["areas"]
    return corr * root, norm * area, dcorr * root[:, None], dnorm * area[:, None]


def correlate_orientations(config, positions, params, bank, residual, fresnel_n=0.0, table=None):
    """correlate for each surfel's own normal and every bank normal, [S, 1 + bank]."""
    corr, norm = kernel.correlate_orientations(
        config, positions, params["centers"], params["normals"], bank, residual, fresnel_n, table
    )
    root = params["areas"].sqrt()[:, None]
    return corr * root, norm * root.square()
