"""The smooth refractive dielectric (raw["material_ior"] / pt_scene_view.
material_ior), an extension of this library: the reference's BSDF has no
refraction, so the oracle's restatement of the Fresnel equations is the
checker, and these CPU tests pin that restatement to physics — energy
conservation in a white furnace, and the reflectance and eta^2 radiance
scaling of a flat interface at normal incidence — and check that the
library's packer and the oracle's carry the indices alike."""
import numpy as np
import pytest

import oracle
import pt_gb300 as P
from pt_gb300 import abi, core, scenes


def test_packers_carry_the_indices():
    raw, cam = scenes.glass_raw("glass")
    hs = P.HostScene.from_raw(raw, cam)
    mine = P.view_arrays(hs.pack())
    assert np.array_equal(mine["material_ior"], raw["material_ior"])
    assert np.array_equal(hs.raw()["material_ior"], raw["material_ior"])
    rs, keep = core.raw_to_struct(raw)
    pk = oracle.OraclePacked(rs)  # owns the arrays its view points to
    theirs = P.view_arrays(pk.view)
    for k in mine:
        assert np.array_equal(np.asarray(mine[k]), np.asarray(theirs[k])), k
    # no indices: a null array, and the scene packs as before
    plain, cam = scenes.tiny_raw("two_tris")
    assert P.view_arrays(P.HostScene.from_raw(plain, cam).pack())["material_ior"].size == 0


@pytest.mark.parametrize("bad", [-1.5, 0.5, np.nan, np.inf])
def test_bad_index_is_rejected(bad):
    raw, cam = scenes.glass_raw("glass")
    raw["material_ior"] = raw["material_ior"].copy()
    raw["material_ior"][2] = bad
    with pytest.raises(P.PtError, match="refraction"):
        P.HostScene.from_raw(raw, cam)
    raw["material_ior"] = raw["material_ior"][:3]
    with pytest.raises(ValueError, match="one entry per material"):
        P.HostScene.from_raw(raw, cam)


def test_white_furnace():
    """A clear glass sphere in a uniform white sky, Russian roulette off:
    reflection and refraction are chosen with the Fresnel probabilities and
    the eta^2 factors cancel on the way out, so every sample carries
    radiance 1 (a path cut by the bounce limit carries 0)."""
    raw, cam = scenes.glass_raw("furnace")
    hs = P.HostScene.from_raw(raw, cam)
    p = hs.render_params(24, 24, 32, 64, rr_start=1000)
    img, _ = oracle.OracleScene(hs.pack()).render(p)
    rgb = img[..., :3]
    assert rgb.max() <= 1.0 + 1e-4
    assert np.mean(np.abs(rgb - 1.0) < 1e-4) > 0.98
    assert abs(float(rgb.mean()) - 1.0) < 2e-3
    # the test discriminates: the same sphere with the reference's BSDF (no
    # index) does not keep the furnace at 1
    raw["material_ior"] = None
    hs2 = P.HostScene.from_raw(raw, cam)
    img2, _ = oracle.OracleScene(hs2.pack()).render(p)
    assert abs(float(img2[..., :3].mean()) - 1.0) > 0.01


def test_flat_interface_at_normal_incidence():
    """Looking straight through one glass quad (index 1.5) at a white sky:
    reflected with F = ((1 - 1.5) / (1 + 1.5))^2 = 0.04 (radiance 1), else
    refracted into the denser side (radiance scaled by (1/1.5)^2) and never
    leaving it, so the mean is F + (1 - F) / 2.25."""
    quad = scenes.quad(50.0, 0.0, True)  # faces down, towards the camera below
    raw = scenes.assemble_raw([(quad, scenes.material_row((1.0, 1.0, 1.0), 0.5), [np.eye(4)])], (1.0, 1.0, 1.0))
    raw["material_ior"] = np.array([1.5], np.float32)
    cam = {"position": (0.0, 5.0, 0.0), "lookdir": (0.0, -1.0, 1e-4), "fov_degrees": 2.0}  # eye at y=-5, looking up
    hs = P.HostScene.from_raw(raw, cam)
    p = hs.render_params(8, 8, 512, 2, rr_start=1000)
    img, _ = oracle.OracleScene(hs.pack()).render(p)
    F = ((1 - 1.5) / (1 + 1.5)) ** 2
    want = F + (1 - F) / 2.25
    assert abs(float(img[..., :3].mean()) - want) < 0.01, (float(img[..., :3].mean()), want)
