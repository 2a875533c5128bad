"""The transforms' tile autotuner: every valid tile width of each pass gives
the same bits (only the block shape changes), and the plan it reports names
a valid width with its timings."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [128, 256])
def test_tile_variants_give_the_same_fields(built, tmp_path, n):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    spec = dict(n_grid=n, z_min=0.05, z_max=0.4, r_smooth=2.0, seed=71, dens_type=1, bias_model=2,
                srcs=[dict(nz=("gauss", 0.2, 0.05), density=10.0, bias=("const", 1.0))])
    prm = cg.Params(inputs.write_inputs(str(tmp_path), spec))
    m = cg.Mock(prm)
    try:
        def grids():
            m.create_cartesian_fields()
            out = [m.grid(0).copy(), m.grid(1).copy()]
            m.compute_physical_density_field()
            return out + [m.grid(w).copy() for w in (2, 3, 4)]
        for p in m.PASSES:
            m.set_field_variant(p, 0)
        ref = grids()
        plan = m.field_plan()
        assert plan["n_grid"] == n
        for p in m.PASSES:
            for v in (1, 2):
                try:
                    m.set_field_variant(p, v)
                except cg.CGError:
                    continue  # not a valid width at this size
                got = grids()
                for a, b in zip(got, ref):
                    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (p, v)
                m.set_field_variant(p, 0)
        for p in m.PASSES:
            m.set_field_variant(p, -1)
        grids()
        plan = m.field_plan()
        print(plan)
        for p in ("fill2", "fill3", "y", "x"):
            assert plan[p]["timed"] or not plan["tuned"]
            tile = [k for k in plan[p] if k not in ("timed", "ms")][0]
            assert plan[p][tile] > 0
            if plan["tuned"]:
                assert str(plan[p][tile]) in plan[p]["ms"]
    finally:
        m.close()
