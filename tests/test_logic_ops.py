"""Comparisons, logic, conditionals, per-element functions and flux-limiter interpolation against the
reference's own outputs (fixtures logic_*: tests/golden/make_golden.py running oracle/_ref/ref_driver).

On a stretched 2D mesh: cell-centred fields c, g, a nodal field v and two velocity fields located at
the targets of the interpolations.  The fixtures hold
  cond     conditional(g > 0., dx<D1FirstOrderBiasedDownwind>(c), dx<D1FirstOrderBiasedUpwind>(c))
  logic    (g > 0.25 && c < 0.5) || !(g >= -0.1)
  exactfn  conditional(g != c, max(c, g) - min(g, c), abs(g)) + sqrt(c) * floor(g * 4.) - ... (exact functions)
  transfn  exp(c) * sin(g) + log(g + 1.5) - pow(c, g + 1.) + ... (transcendental functions)
  fx_<K>   d1Intp<0, Cen2Cor, D1FluxLimiterGen<K>::Op>(ux, c) for all 17 limiter kernels
  fy_<K>   d1Intp<1, Cor2Cen, D1FluxLimiterGen<K>::Op>(uy, v)
The oracle matches every dump bit for bit, NaN where the reference has NaN (a limiter's slope ratio
r = slope_f / (slope_u + 1e-16) is 0/0 or inf/inf where the field is flat next to a boundary).  The
CUDA library matches every dump bit for bit except transfn, whose CUDA math functions differ from the
host C library's by a few ulp: |got - want| <= 1e-14 + 4e-15 |want| (values of order 1 to 10).
"""
import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

CASES = ["logic_12x9", "logic_16x20"]
LIMITERS = ["CDS", "QUICK", "CUI", "Fromm", "LUI", "Minmod", "Superbee", "MUSCL", "Harmonic", "vanAlbada", "UMIST",
            "SPL13", "SPLMax12", "SPLMax13", "Koren", "SMART", "BSOU"]
TRANS_RTOL, TRANS_ATOL = 4e-15, 1e-14


def _desc(l0, l1, periodic_y):
    bc_x_end = capi.BC_DIRC if (l0 == capi.CORNER and l1 == capi.CENTER) else capi.BC_NEUM
    val_x_end = -1.0
    bcs = [(capi.BC_DIRC, bc_x_end), (capi.BC_PERIODIC, capi.BC_PERIODIC) if periodic_y else (capi.BC_NEUM, capi.BC_DIRC)]
    vals = [(0.5, val_x_end), (0.0, 0.0) if periodic_y else (0.0, 1.0)]
    return cm.field_desc(2, [l0, l1], bcs, vals, ext=1)


DESCS = {
    "c": _desc(capi.CENTER, capi.CENTER, True),
    "g": _desc(capi.CENTER, capi.CENTER, True),
    "v": _desc(capi.CORNER, capi.CORNER, False),
    "ux": _desc(capi.CORNER, capi.CENTER, True),
    "uy": _desc(capi.CORNER, capi.CENTER, False),
}
SEED_OFF = {"c": (0, 0.0), "g": (1, 0.5), "v": (2, 0.25), "ux": (3, 0.5), "uy": (4, 0.5)}


def _case(name):
    meta, arr = cm.golden(name)
    _, nx, ny, seed = meta["args"]
    nx, ny, seed = int(nx), int(ny), int(seed)
    mesh = cm.mesh_points([cm.stretched_points(nx + 1), cm.stretched_points(ny + 1, 2.0)])
    hosts = {}
    for key, fd in DESCS.items():
        hf = orc.HostField(mesh, fd)
        rng = hf.assignable()
        j, i = np.meshgrid(np.arange(*rng[1]), np.arange(*rng[0]), indexing="ij")
        s, shift = SEED_OFF[key]
        hf.data[hf.slices(rng)] = orc.u01(seed + s, j.astype(np.uint64) * np.uint64(1000) + i.astype(np.uint64)) - shift
        hf.update_padding()
        hosts[key] = hf
    return meta, arr, mesh, hosts


def _outputs(F):
    """(key, destination desc, expression) over the leaves F[c, g, v, ux, uy]."""
    c, g, v, ux, uy = F["c"], F["g"], F["v"], F["ux"], F["uy"]
    out = [
        ("cond", DESCS["c"], api.conditional(g > 0., api.dx(c, api.D1FirstOrderBiasedDownwind),
                                             api.dx(c, api.D1FirstOrderBiasedUpwind))),
        ("logic", DESCS["c"], ((g > 0.25) & (c < 0.5)) | ~(g >= -0.1)),
        ("exactfn", DESCS["c"], api.conditional(g != c, api.max(c, g) - api.min(g, c), api.abs(g))
         + api.sqrt(c) * api.floor(g * 4.) - api.ceil(c * 3.) + api.round(g * 7.) + api.trunc(c * 5.)
         + api.fdim(c, g) + api.copysign(c, g) + api.fmod(c * 7., g + 1.)),
        ("transfn", DESCS["c"], api.exp(c) * api.sin(g) + api.log(g + 1.5) - api.pow(c, g + 1.) + api.tanh(g)
         + api.atan2(g, c) + api.hypot(c, g) + api.erf(g) + api.cbrt(g) + api.log1p(c) + api.expm1(g) + api.cos(c)
         + api.sqrt(c * c + g * g)),
    ]
    for k, name in enumerate(LIMITERS):
        out.append(("fx_" + name, DESCS["ux"], api.d1_flux_limiter_intp(ux, c, 0, k, to_corner=True)))
        out.append(("fy_" + name, DESCS["uy"], api.d1_flux_limiter_intp(uy, v, 1, k, to_corner=False)))
    return out


def _readable(hf):
    return hf.data[hf.slices(cm.readable(hf.info))].reshape(-1)


def test_limiter_names_follow_the_enum():
    assert [api.FLUX_LIMITERS[n] for n in ["Central", "QUICK", "CUI", "Fromm", "LinearUpwind", "Minmod", "Superbee",
                                           "MUSCL", "Harmonic", "Albada", "UMIST", "SPL13", "SPLMax12", "SPLMax13",
                                           "KorenLimitedCUI", "SMART", "BSOU"]] == list(range(17))


@pytest.mark.parametrize("name", CASES)
def test_logic_and_limiters_oracle_bitexact(name):
    meta, arr, mesh, hosts = _case(name)
    for key in DESCS:
        assert np.array_equal(_readable(hosts[key]), arr[key + "__data"]), key
    L = {k: cm.Leaf(k) for k in DESCS}
    order = [L[k] for k in DESCS]
    for key, fd, expr in _outputs(L):
        out = orc.HostField(mesh, fd)
        nodes, _ = api.serialize(expr, order)
        orc.assign(out, nodes, [hosts[k] for k in DESCS] + [out])
        assert np.array_equal(_readable(out), arr[key + "__data"], equal_nan=True), key


def test_reference_kernels_use_integer_ratio_parameters():
    """SPLMinKernel<2, 1/2> and <2, 1/3> coincide in the reference (its m and kappa divide the ratio's
    integers), and so they do here."""
    meta, arr = cm.golden("logic_12x9")
    assert np.array_equal(arr["fx_UMIST__data"], arr["fx_SPL13__data"])
    assert np.array_equal(arr["fx_SPLMax12__data"], arr["fx_SPLMax13__data"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_logic_and_limiters_gpu_match_reference_dump(ctx, name):
    meta, arr, mesh, hosts = _case(name)
    F = {}
    for key, fd in DESCS.items():
        F[key] = api.CartesianField(mesh, fd, ctx)
        F[key].upload(hosts[key].data, update_padding=False)
    for key, fd, expr in _outputs(F):
        out = api.CartesianField(mesh, fd, ctx)
        out.assign(expr)
        got = out.download()[out.index_slices(cm.readable(out.info))].reshape(-1)
        want = arr[key + "__data"]
        if key == "transfn":
            np.testing.assert_allclose(got, want, rtol=TRANS_RTOL, atol=TRANS_ATOL, err_msg=key)
        else:
            assert np.array_equal(got, want, equal_nan=True), key
