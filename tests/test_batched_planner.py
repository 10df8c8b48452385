"""The batched CG's planner (host logic, no device): which kernel variant a launch over the running instances gets
and how many CTAs each instance is given, on given co-resident capacities."""
import numpy as np
import pytest

import ikarus_gb300 as ikr

CAPS = (456, 304, 304, 304, 0, 304)  # co-resident CTAs of variants 0..5 on a 152-SM device (3, 2, 2, 2, -, 2 per SM)


def plan(rows, fp32=True, variant=-1, widths=None, caps=CAPS, cluster_cap=7):
    w = [27] * len(rows) if widths is None else widths
    return ikr.batched_plan_preview(rows, w, fp32, variant, caps, cluster_cap)


def test_fp32_small_instances_get_one_cluster_each():
    v, c = plan([297, 60, 425])
    assert v == 4 and (c == 16).all()


def test_fp32_large_instances_get_eight_threads_per_row():
    """The cluster variant is the planner's choice only up to 512 rows; beyond, 32 rows per CTA."""
    v, c = plan([2673])
    assert v == 3 and c.tolist() == [-(-2673 // 32)]
    v, c = plan([2673], variant=4)  # forced, it still fits one cluster (at most 16 x 192 rows)
    assert v == 4


def test_more_instances_than_clusters_fall_back_to_shared_memory_groups():
    v, c = plan([100] * 8)
    assert v == 3 and (c == 4).all()


def test_fp64_prefers_sixteen_threads_per_row_for_small_groups_only():
    v, c = plan([297], fp32=False)
    assert v == 5 and c.tolist() == [-(-297 // 16)]
    v, c = plan([2673], fp32=False)  # 168 CTAs at sixteen threads per row: more than 64, so eight
    assert v == 3 and c.tolist() == [-(-2673 // 32)]


def test_groups_that_do_not_fit_the_device_fall_back_to_the_row_loop():
    rows = [2500] * 20  # 20 x 79 CTAs at eight threads per row > 304; 20 x 40 at four > 304; 20 x 10 at one row per thread fits
    v, c = plan(rows)
    assert v == 1 and (c == 10).all()
    rows = [2500] * 40  # one row per thread: 400 CTAs > 304 -> the row loop with the smallest rows per CTA that fits
    v, c = plan(rows)
    assert v == 0 and c.sum() <= CAPS[0] and (c >= 1).all()
    q = -(-2500 // c[0])
    assert c[0] == min(-(-2500 // q), 2500 // 64, 32)


def test_more_instances_than_resident_ctas_run_one_cta_each():
    v, c = plan([300] * 500)
    assert v == 0 and (c == 1).all()


def test_wide_slices_skip_the_shared_memory_variants():
    """A slice wider than a shared-memory variant holds (eight threads x four blocks) goes to one row per thread."""
    v, c = plan([200], widths=[40], cluster_cap=0)
    assert v == 1


def test_a_forced_variant_that_does_not_fit_falls_back_to_the_row_loop():
    v, c = plan([2500] * 20, variant=3)
    assert v == 0


@pytest.mark.parametrize("fp32", [True, False])
def test_invalid_arguments(fp32):
    with pytest.raises(ikr.IkarusError, match="ARG"):
        ikr.batched_plan_preview([100], [27], fp32, 7, CAPS, 7)
