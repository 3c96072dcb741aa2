"""Consistency of the oracle's BSDF restatement (pt_oracle.c, the
reference's DiffuseBxDF and GlossyBxDF with its GGX distribution) on CPU:
the sampling pdf is a density over the directions (integrates to 1, or to
less for GGX whose reflected directions may fall below the surface),
Lambert's eval / pdf is its albedo, and no lobe reflects more energy than
it receives.  The images these BSDFs make are pinned to the reference bit
for bit (test_oracle_pins.py); this checks the math they restate."""
import numpy as np
import pytest


def _sphere(n, seed=3):
    rng = np.random.default_rng(seed)
    z = rng.uniform(-1, 1, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    r = np.sqrt(1 - z * z)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], -1).astype(np.float32)


def _eval(kind, rough, wo, wi, albedo=0.5):
    from oracle.oracle import bsdf_eval
    n = len(wi)
    params = np.tile(np.array([kind, albedo, albedo, albedo, rough, 1.5], np.float32), (n, 1))
    normal = np.tile(np.array([0, 0, 1], np.float32), (n, 1))
    tangent = np.tile(np.array([1, 0, 0], np.float32), (n, 1))
    return bsdf_eval(params, normal, tangent, np.tile(np.asarray(wo, np.float32), (n, 1)), wi)


def test_lambert_pdf_and_weight():
    wi = _sphere(200_000)
    ev, pdf, nz = _eval(0, 0.3, [0.0, 0.6, 0.8], wi)
    assert np.mean(pdf * nz) * 4 * np.pi == pytest.approx(1.0, abs=0.01)
    up = nz.astype(bool)
    assert np.allclose(ev[up, 0] / pdf[up], 0.5, rtol=1e-5)  # f cos / pdf = albedo


@pytest.mark.parametrize("rough", [0.3, 0.6])
@pytest.mark.parametrize("wo", [[0.0, 0.0, 1.0], [0.866, 0.0, 0.5]])
def test_ggx_pdf_is_a_density_and_energy_is_bounded(rough, wo):
    wi = _sphere(400_000, seed=7)
    ev, pdf, nz = _eval(1, rough, wo, wi)
    mass = float(np.mean(pdf * nz) * 4 * np.pi)
    assert 0.8 < mass < 1.02, mass
    albedo = float(np.mean(ev[:, 0] * nz) * 4 * np.pi)  # integral of f cos over the directions
    assert 0.0 < albedo < 1.02, albedo
