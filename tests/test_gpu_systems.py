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
