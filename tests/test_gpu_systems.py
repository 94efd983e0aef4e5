"""Uneven multi-system batches: each system's logL from the persistent
multi-system launch equals its own single-system context's (same per-pixel
arithmetic and summation orders), for changing per-call counts."""
import numpy as np
import pytest

import lensed_gb300 as lg
from lensed_gb300 import workloads

pytestmark = pytest.mark.gpu


def _systems(n=6):
    out = workloads.systems(count=n)
    return out


def test_systems_match_single_contexts(native):
    syst = _systems(6)
    objs = syst[0].objects
    S = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], objs, capacity=[8] * len(syst), rule="g3k7")
    for call, counts in enumerate(([8, 3, 0, 5, 8, 1], [2, 8, 7, 0, 1, 4])):
        params = []
        for s, c in zip(syst, counts):
            ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=8)
            params.append(ctx.to_map_order(workloads.draw_candidates(s, c, seed=call)))
            ctx.close()
        got = S.eval(params)
        for s, p, g in zip(syst, params, got):
            if len(p) == 0:
                assert g.size == 0
                continue
            ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=8)
            want = ctx.eval_batch(p)
            assert np.array_equal(g, want), (s.name, g - want)
            ctx.close()


def test_systems_reject_bad_counts(native):
    syst = _systems(2)
    S = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], syst[0].objects, capacity=[2, 2])
    with pytest.raises(lg.LensedError):
        S.eval([np.zeros((3, S.npars)), np.zeros((1, S.npars))])


def test_systems_with_paired_and_single_row_units(native):
    """PSFs on both sides of the paired-row limit (49 pixels) in one batch:
    each system still equals its own context, in every mode."""
    base = _systems(3)
    widths = [15, 51, 25]
    syst = []
    for s, w in zip(base, widths):
        psf = workloads.psf_gauss_wings(w, 2.0)
        syst.append((s, psf))
    objs = base[0].objects
    for flags in (0, lg.LG_FLAG_STRICT_FP, lg.LG_FLAG_FAST_MATH):
        S = lg.Systems([(s.image, s.weight, psf, None) for s, psf in syst], objs, capacity=[3] * 3, rule="g3k7",
                       flags=flags)
        params = []
        for s, psf in syst:
            ctx = lg.Context(s.image, s.weight, s.objects, psf=psf, rule="g3k7", max_batch=3, flags=flags)
            params.append(ctx.to_map_order(workloads.draw_candidates(s, 3, seed=5)))
            ctx.close()
        got = S.eval(params)
        for (s, psf), p, g in zip(syst, params, got):
            ctx = lg.Context(s.image, s.weight, s.objects, psf=psf, rule="g3k7", max_batch=3, flags=flags)
            assert np.array_equal(g, ctx.eval_batch(p)), (s.name, flags)
            ctx.close()


@pytest.mark.parametrize("flags", [0, lg.LG_FLAG_FAST_MATH])
def test_systems_full_size_against_the_oracle(native, flags):
    """The uneven multi-system workload at full size (16 systems of 64^2 to
    512^2, EPL + shear with slopes t in [0.8, 1.2], Sersic, sky, odd PSFs of
    15 to 31 pixels, 49-point g3k7 rule), two candidates per system through
    the persistent multi-system launch, against the FP32 oracle of each
    system: |dlogL| <= 1e-3 in the default (exact) mode, the fast mode's
    widened bound 1e-3 + 2e-6 |logL| with LG_FLAG_FAST_MATH; the distance to
    the FP64 oracle is printed."""
    from lensed_gb300 import quadrature
    from oracle.oracle import Oracle

    syst = workloads.systems()
    S = lg.Systems([(s.image, s.weight, s.psf, None) for s in syst], syst[0].objects, capacity=[2] * len(syst),
                   rule="g3k7", flags=flags)
    cands, params = [], []
    for k, s in enumerate(syst):
        ctx = lg.Context(s.image, s.weight, s.objects, psf=s.psf, rule=s.rule, max_batch=2, flags=flags)
        c = workloads.draw_candidates(s, 2, seed=40 + k)
        cands.append(c)
        params.append(ctx.to_map_order(c))
        ctx.close()
    got = S.eval(params)
    worst = 0.0
    for s, c, g in zip(syst, cands, got):
        kw = dict(psf=s.psf, image=s.image, weight=s.weight, threads=16)
        w32 = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), precision=32, **kw).loglike(c)
        w64 = Oracle(s.plugins, s.width, s.height, quadrature.rule(s.rule), precision=64, **kw).loglike(c)
        d = np.abs(g - w32)
        tol = 1e-3 if not flags else 1e-3 + 2e-6 * np.abs(w32)
        print(f"{s.name}: |dlogL| vs FP32 oracle {np.array2string(d, precision=2)}, vs FP64 "
              f"{np.array2string(np.abs(g - w64), precision=2)}, FP32 oracle vs FP64 "
              f"{np.array2string(np.abs(w32 - w64), precision=2)}")
        assert np.all(d <= tol), (s.name, d)
        worst = max(worst, d.max())
    print(f"16 systems, {'fast' if flags else 'exact'} mode: max |dlogL| vs FP32 oracle {worst:.3g}")
