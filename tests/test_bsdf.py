"""The oracle's Principled BSDF on CPU (double precision): the full model the
renderer uses for `Principled` materials (scenes/cbox.json:3-62) — Lambert,
sheen, GGX with specular tint, a rough dielectric glass lobe and a GTR1
clearcoat. Every check here is a property of the mathematics, not of an
implementation:

- the sampler draws directions with the density the pdf function reports
  (binned chi-square over the sphere, refraction included);
- the estimator f |cos| / pdf of sampled directions averages to the
  quadrature of f |cos| over the sphere (sampling, pdf and eval agree);
- reflection is reciprocal, and refraction obeys the generalised
  reciprocity of radiance BTDFs: f(wo, wi; eta) * eta^2 = f(wi', wo'; 1/eta)
  with both directions mirrored through the surface;
- reflection-only materials and glass entered from outside do not create
  energy (albedo <= 1);
- with sheen, clearcoat, specular tint and transmission all 0 the full model
  equals the Lambert + GGX base model of the reference scenes.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import aqua
import pyoracle


def material(**kw) -> aqua.Material:
    m = aqua.Material()
    m.base_color[:] = kw.pop("color", (0.8, 0.6, 0.4))
    m.base_texture = -1
    defaults = dict(metallic=0.0, roughness=0.5, specular=0.5, specular_tint=0.0, sheen=0.0, sheen_tint=0.5,
                    clearcoat=0.0, clearcoat_roughness=0.03, transmission=0.0, ior=1.45)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(m, k, v)
    return m


MATERIALS = {
    "lambert": material(specular=0.0),
    "ggx_dielectric": material(roughness=0.3),
    "ggx_metal": material(metallic=1.0, roughness=0.4),
    "tinted_specular": material(specular=1.0, specular_tint=1.0, roughness=0.35),
    "sheen": material(sheen=1.0, sheen_tint=0.7, roughness=0.8),
    "clearcoat": material(clearcoat=1.0, clearcoat_roughness=0.3, roughness=0.6),
    "glass": material(transmission=1.0, roughness=0.5, color=(1.0, 1.0, 1.0)),
    "frosted_mix": material(transmission=0.6, metallic=0.2, roughness=0.5, clearcoat=0.5, clearcoat_roughness=0.3,
                            sheen=0.4),
}


def unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def sphere_grid(n_ct: int, n_phi: int):
    """Midpoints of an equal-area grid over the whole sphere (cos theta
    uniform in [-1, 1]); returns (directions, solid angle per cell)."""
    ct = -1.0 + (np.arange(n_ct) + 0.5) * (2.0 / n_ct)
    ph = (np.arange(n_phi) + 0.5) * (2 * np.pi / n_phi)
    C, P = np.meshgrid(ct, ph, indexing="ij")
    s = np.sqrt(1 - C * C)
    d = np.stack([s * np.cos(P), s * np.sin(P), C], axis=-1).reshape(-1, 3)
    return d, 4 * np.pi / (n_ct * n_phi)


WO = [unit(np.array([0.3, 0.1, 0.9])), unit(np.array([-0.6, 0.2, 0.35])), unit(np.array([0.05, -0.8, 0.2]))]


CHI_CASES = [(n, True) for n in sorted(MATERIALS)] + \
    [(n, False) for n in sorted(MATERIALS) if MATERIALS[n].transmission > 0]  # back side: glass only


@pytest.mark.parametrize("name,front", CHI_CASES)
def test_sampling_matches_pdf_chi_square(name, front):
    m = MATERIALS[name]
    rng = np.random.default_rng(7)
    n_ct, n_phi, sub = 24, 48, 16
    for wo in WO[:2]:
        N = 300_000
        wi = pyoracle.bsdf_sample(m, wo[None, :], rng.random((N, 3)), front=front)
        ok = wi[:, 2] != 0.0
        _, p = pyoracle.bsdf_eval(m, wo[None, :], np.where(ok[:, None], wi, [[0, 0, 1.0]]), front=front)
        ok &= p > 0  # samples the pdf does not cover carry no weight
        wi = unit(wi[ok])
        ib = np.clip(((wi[:, 2] + 1) / 2 * n_ct).astype(int), 0, n_ct - 1)
        jb = np.clip(((np.arctan2(wi[:, 1], wi[:, 0]) % (2 * np.pi)) / (2 * np.pi) * n_phi).astype(int), 0,
                     n_phi - 1)
        obs = np.bincount(ib * n_phi + jb, minlength=n_ct * n_phi).astype(np.float64)
        # expected counts: the pdf integrated over each cell (sub x sub midpoints)
        d, dw = sphere_grid(n_ct * sub, n_phi * sub)
        _, pd = pyoracle.bsdf_eval(m, wo[None, :], d, front=front)
        cell = pd.reshape(n_ct, sub, n_phi, sub).sum(axis=(1, 3)) * dw
        exp = N * cell.reshape(-1)
        mask = exp > 25
        chi2 = np.sum((obs[mask] - exp[mask]) ** 2 / exp[mask])
        dof = mask.sum() - 1
        assert chi2 / dof < 1.6, (name, front, chi2 / dof)
        # the pdf integrates to the fraction of valid samples
        assert abs(cell.sum() - ok.mean()) < 0.01, (name, cell.sum(), ok.mean())


@pytest.mark.parametrize("name", sorted(MATERIALS))
def test_estimator_equals_quadrature(name):
    m = MATERIALS[name]
    rng = np.random.default_rng(11)
    d, dw = sphere_grid(800, 1600)
    for wo in WO:
        f, _ = pyoracle.bsdf_eval(m, wo[None, :], d)
        quad = (f * np.abs(d[:, 2:3])).sum(axis=0) * dw
        N = 400_000
        wi = pyoracle.bsdf_sample(m, wo[None, :], rng.random((N, 3)))
        ok = wi[:, 2] != 0.0
        wi = np.where(ok[:, None], wi, [[0, 0, 1.0]])
        fs, ps = pyoracle.bsdf_eval(m, wo[None, :], wi)
        w = np.where((ok & (ps > 0))[:, None], fs * np.abs(wi[:, 2:3]) / np.where(ps > 0, ps, 1)[:, None], 0.0)
        est = w.mean(axis=0)
        se = w.std(axis=0) / np.sqrt(N)
        np.testing.assert_array_less(np.abs(est - quad), 5 * se + 3e-3 * quad + 1e-4, err_msg=name)


@pytest.mark.parametrize("name", sorted(MATERIALS))
def test_reflection_is_reciprocal(name):
    m = MATERIALS[name]
    rng = np.random.default_rng(3)
    a = unit(rng.normal(size=(2000, 3)) * [1, 1, 0] + [0, 0, 0.05] + np.abs(rng.normal(size=(2000, 1))) * [0, 0, 1])
    b = unit(rng.normal(size=(2000, 3)) * [1, 1, 0] + [0, 0, 0.05] + np.abs(rng.normal(size=(2000, 1))) * [0, 0, 1])
    fab, _ = pyoracle.bsdf_eval(m, a, b)
    fba, _ = pyoracle.bsdf_eval(m, b, a)
    np.testing.assert_allclose(fab, fba, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("ior", [1.33, 1.45, 2.0])
@pytest.mark.parametrize("front", [True, False])
def test_refraction_generalised_reciprocity(ior, front):
    m = material(transmission=1.0, roughness=0.35, ior=ior, color=(1.0, 1.0, 1.0))
    ior = float(m.ior)  # as stored (float32)
    eta = ior if front else 1.0 / ior
    rng = np.random.default_rng(5)
    wo = unit(rng.normal(size=(4000, 3)) * [1, 1, 0.6] + [0, 0, 0.5])
    wo[:, 2] = np.abs(wo[:, 2]) + 1e-3
    wo = unit(wo)
    wi = unit(rng.normal(size=(4000, 3)) * [1, 1, 0.6] - [0, 0, 0.5])
    wi[:, 2] = -np.abs(wi[:, 2]) - 1e-3
    wi = unit(wi)
    f, _ = pyoracle.bsdf_eval(m, wo, wi, front=front)
    flip = np.array([1.0, 1.0, -1.0])
    g, _ = pyoracle.bsdf_eval(m, wi * flip, wo * flip, front=not front)
    assert (f[:, 0] > 0).mean() > 0.1  # enough pairs are valid refraction pairs
    np.testing.assert_allclose(g, f * eta * eta, rtol=1e-8, atol=1e-12)


SINGLE_LOBES = {
    "lambert": material(specular=0.0, color=(1.0, 1.0, 1.0)),
    "ggx_metal": material(metallic=1.0, roughness=0.4, color=(1.0, 1.0, 1.0)),
    "clearcoat_only": material(clearcoat=1.0, clearcoat_roughness=0.2, specular=0.0, color=(0.0, 0.0, 0.0)),
    "glass": material(transmission=1.0, roughness=0.5, color=(1.0, 1.0, 1.0)),
    "glass_rough": material(transmission=1.0, roughness=0.9, color=(1.0, 1.0, 1.0)),
}


@pytest.mark.parametrize("name", sorted(SINGLE_LOBES))
def test_albedo_at_most_one(name):
    """Single lobes do not create energy (diffuse + specular of the additive
    Principled model may exceed 1 at grazing angles by construction, so the
    lobes are checked one at a time; glass is entered from outside)."""
    m = SINGLE_LOBES[name]
    d, dw = sphere_grid(600, 1200)
    for wo in WO + [unit(np.array([0.0, 0.999, 0.03]))]:
        f, _ = pyoracle.bsdf_eval(m, wo[None, :], d, front=True)
        albedo = (f * np.abs(d[:, 2:3])).sum(axis=0) * dw
        assert np.all(albedo <= 1.0 + 2e-3), (name, albedo)


def test_full_model_reduces_to_the_base_model():
    """With the extra lobes at 0 the full model is Lambert + GGX: compare with
    an independent evaluation of (1-m) C / pi + F D G2 / (4 cos cos)."""
    rng = np.random.default_rng(9)
    for metallic, rough, spec in [(0.0, 0.5, 0.5), (1.0, 0.2, 0.0), (0.3, 0.9, 1.0)]:
        m = material(metallic=metallic, roughness=rough, specular=spec, ior=1.7, clearcoat_roughness=0.4)
        metallic, rough, spec = float(m.metallic), float(m.roughness), float(m.specular)  # as stored (float32)
        wo = unit(np.abs(rng.normal(size=(500, 3))) * [1, 1, 1] + [0, 0, 0.1])
        wi = unit(rng.normal(size=(500, 3)) * [1, 1, 0] + np.abs(rng.normal(size=(500, 1))) * [0, 0, 1] + [0, 0, 0.05])
        f, _ = pyoracle.bsdf_eval(m, wo, wi)
        C = np.array(m.base_color[:])
        a2 = max(rough * rough, 1e-3) ** 2
        h = unit(wo + wi)
        D = a2 / (np.pi * (h[:, 2] ** 2 * (a2 - 1) + 1) ** 2)
        lam = lambda c: 0.5 * (-1 + np.sqrt(1 + a2 * (1 - c * c) / (c * c)))
        G2 = 1 / (1 + lam(wo[:, 2]) + lam(wi[:, 2]))
        F0 = 0.08 * spec + (C - 0.08 * spec) * metallic
        F = F0 + (1 - F0) * np.clip(1 - np.sum(wi * h, axis=1), 0, 1)[:, None] ** 5
        expect = (1 - metallic) * C / np.pi + (F if (0.08 * spec * 3 + metallic) > 0 else 0) * \
            (D * G2 / (4 * wo[:, 2] * wi[:, 2]))[:, None]
        np.testing.assert_allclose(f, expect, rtol=1e-9, atol=1e-12)


def test_principled_scene_lobes_are_loaded_and_change_the_image(host_ctx, tmp_path):
    """The reference's cbox.json with glass, clearcoat, sheen and tinted
    specular materials (the GPU test's scene) loads with those parameters,
    renders finite, and differs from the unedited scene."""
    import json

    from conftest import reference_scene
    from test_gpu_principled import EDITS, principled_scene

    s = host_ctx.load_scene(principled_scene(tmp_path))
    mats = s.materials()
    assert sorted(round(m.transmission, 3) for m in mats if m.transmission > 0) == [0.3, 1.0]
    assert max(m.clearcoat for m in mats) == 1.0 and max(m.sheen for m in mats) == 1.0
    assert max(m.specular_tint for m in mats) == 1.0
    o = pyoracle.OracleScene.from_aqua(s)
    o.set_resolution(32, 32)
    img, st = o.render(16, 8, seed=2, precision=32)
    base = host_ctx.load_scene(reference_scene("cbox.json"))
    ob = pyoracle.OracleScene.from_aqua(base)
    ob.set_resolution(32, 32)
    ref, _ = ob.render(16, 8, seed=2, precision=32)
    assert np.isfinite(img).all() and img.mean() > 0.01
    assert pyoracle.rel_mse(img, ref) > 1e-2
    s.free()
    base.free()
    # parameters outside their ranges are refused
    d = json.load(open(reference_scene("cbox.json")))
    for key, bad in (("ior", 0.5), ("sheen", 1.5), ("transmission", -0.1), ("clearcoat_roughness", 2.0)):
        e = json.loads(json.dumps(d))
        e["named_bsdfs"]["floor"]["Principled"][key] = {"Float": bad}
        for shape in e["shapes"]:
            shape["Mesh"][0] = os.path.join(os.path.dirname(reference_scene("cbox.json")), shape["Mesh"][0])
        p = tmp_path / f"bad_{key}.json"
        p.write_text(json.dumps(e))
        with pytest.raises(aqua.AquaError) as err:
            host_ctx.load_scene(str(p))
        assert err.value.status == aqua.ERR_PARSE and key in str(err.value)
