"""FLOP/byte model: einsum counts follow the reference's counting rule."""

import numpy as np
import pytest

from actx_dgfem_suite_gb300 import perf_model as pm


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_einsum_counts_match_opt_einsum(order):
    oe = pytest.importorskip("opt_einsum")
    from math import prod
    E = 7
    n, nfp = pm.np_of(order), pm.nfp_of(order)

    def count(spec, shapes):
        ops = [np.empty(s) for s in shapes]
        _, info = oe.contract_path(spec, *ops, optimize="optimal", use_blas=False)
        tot = 0
        for (_, contracted, es, _, _) in info.contraction_list:
            it = prod(info.size_dict[c]
                      for c in set(es.translate(str.maketrans("", "", " ->,"))))
            tot += 2 * it if contracted else it
        return tot // E

    assert count("re,rji,ej->ei", [(3, E), (3, n, n), (E, n)]) == pm.grad_flops(order)
    assert count("xre,rji,xej->ei", [(3, 3, E), (3, n, n), (3, E, n)]) \
        == pm.div_flops(order)
    assert count("jfi,fe,fej->ei", [(nfp, 4, n), (4, E), (4, E, nfp)]) \
        == pm.lift_flops(order)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_einsum_counts_match_opt_einsum_2d(order):
    """Triangles: two reference axes, three edges."""
    oe = pytest.importorskip("opt_einsum")
    from math import prod
    E = 7
    n, nfp = pm.np_of(order, 2), pm.nfp_of(order, 2)

    def count(spec, shapes):
        ops = [np.empty(s) for s in shapes]
        _, info = oe.contract_path(spec, *ops, optimize="optimal", use_blas=False)
        tot = 0
        for (_, contracted, es, _, _) in info.contraction_list:
            it = prod(info.size_dict[c]
                      for c in set(es.translate(str.maketrans("", "", " ->,"))))
            tot += 2 * it if contracted else it
        return tot // E

    assert count("re,rji,ej->ei", [(2, E), (2, n, n), (E, n)]) == pm.grad_flops(order, 2)
    assert count("xre,rji,xej->ei", [(2, 2, E), (2, n, n), (2, E, n)]) \
        == pm.div_flops(order, 2)
    assert count("jfi,fe,fej->ei", [(nfp, 3, n), (3, E), (3, E, nfp)]) \
        == pm.lift_flops(order, 2)
    c = pm.RhsCost("euler", order, 10, dim=2)
    assert c.dofs == 4 * 10 * n and c.flops > 0 and c.bytes > 0


def test_known_values():
    assert [pm.grad_flops(p) for p in (1, 2, 3, 4)] == [108, 630, 2460, 7455]
    assert [pm.div_flops(p) for p in (1, 2, 3, 4)] == [168, 780, 2760, 7980]
    assert [pm.lift_flops(p) for p in (1, 2, 3, 4)] == [108, 504, 1640, 4260]


def test_cost_object():
    c = pm.RhsCost("wave", 3, 1000)
    assert c.dofs == 4 * 1000 * 20
    assert c.bytes == 1000 * (16 * 4 * 20 + 72 + 128 + 16 * 10)
    assert c.roofline_seconds(1e12, 1e12) == max(c.flops, c.bytes) / 1e12


def test_wave_pointwise_counts_follow_the_reference_code():
    """The wave equation's pointwise counts are those of the reference's own
    wave_operator, counted on stand-ins (tests/golden/make_reference_flop_counts.py)."""
    import json
    from pathlib import Path
    fx = json.loads((Path(__file__).parent / "golden" / "reference_wave_flops.json").read_text())
    for key, table in (("orders", pm._POINTWISE), ("orders_2d", pm._POINTWISE_2D)):
        face, vol = table["wave"]
        for order, c in fx[key].items():
            assert c["per_node"] == vol
            assert c["per_interior_face_point"] + c["per_all_faces_point"] == face
            assert c["per_boundary_face_point"] - c["per_interior_face_point"] \
                == pm.WAVE_BOUNDARY_EXTRA
    n, order = 3, 2
    c = pm.RhsCost("wave", order, 6 * n**3, boundary_faces=12 * n * n)
    assert c.flops == 6 * n**3 * pm.flops_per_element("wave", order) + 12 * n * n * pm.nfp_of(order)


def test_print_roofline_dims_2_and_3(capsys):
    from actx_dgfem_suite_gb300.tools.print_roofline import main
    rows = main(["--equations", "tiny_wave,euler", "--dims", "2,3", "--degrees", "1,4"])
    assert {(r[0], r[1], r[2]) for r in rows} == {
        (dim, eq, d) for dim in (2, 3) for eq in ("tiny_wave", "euler") for d in (1, 4)}
    assert all(r[4] > 0 and r[5] > 0 and r[6] > 0 for r in rows)
    assert " 2 euler" in capsys.readouterr().out
