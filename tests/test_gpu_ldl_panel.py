"""The LDL^T variants (the column kernel and panels of 2, 4, 8 columns
broadcast over the cluster), on 16- or 8-CTA clusters, give the same factors
bit for bit: every column receives the same updates in the same order with
the same FMAs.  Checked
through whole frames (the fit's solution and the difference image), each
variant forced with option "tune_variant" (which also picks the conv's tile
shape, whose variants are identical too)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("size,n_src,stamps", [(1024, 5000, 16), (2048, 20000, 16), (512, 1500, 10)])
def test_ldl_variants_agree(size, n_src, stamps):
    import xbach
    from xbach.synth import make_pair
    T, S, info = make_pair(2, frame=3, size=size, n_src=n_src, stamps=stamps)
    p = xbach.default_params(mode=xbach.XB_MODE_MIXED, stampsx=stamps, stampsy=stamps,
                             threshHigh=info["threshHigh"])
    out = []
    for variant in (0, 1, 2, 3, -1, -8):
        ctx = xbach.Context(p)
        if variant == -1:
            ctx.set_option("ldl_panel", 0)
        elif variant == -8:  # an 8-CTA cluster instead of 16
            ctx.set_option("ldl_cluster", 8)
        else:
            ctx.set_option("tune_variant", variant)
        ctx.run_all(T, S)
        out.append((ctx.solution(), ctx.image(xbach.XB_IMG_DIFF, f64=False),
                    ctx.scalar("ksc_iterations")))
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0])
        assert np.array_equal(out[0][1], o[1])
        assert out[0][2] == o[2]
