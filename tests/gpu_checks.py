"""Checks shared by the GPU parity tests: the CUDA pipeline, through the C
ABI, against the CPU oracle at every stage (bit for bit)."""
import numpy as np

import bdcudatag
import oracle


def kat_config(**kw):
    return bdcudatag.default_config(max_detections=32, min_decision_margin=2.0, **kw)


def okat_config(**kw):
    return oracle.default_config(max_detections=32, min_decision_margin=2.0, **kw)


def same_records(a, b):
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (a, b)


# FrameState as uint32 words: counts[5], top_enc, bottom_enc, ref[2],
# done_stats, done_cands, n_candidates, n_big, n_small, span_hist[256],
# mean_hist[64], bin_base[64].
STATE_REF = slice(7, 9)
STATE_SPAN = slice(14, 14 + 256)
STATE_MEAN = slice(270, 270 + 64)


def check_tile_stats(tile_min, tile_max, state, ref):
    """The first stage against the oracle: tile extremes, both histograms
    and the two frame references (noise-floor quartile, Otsu level)."""
    assert np.array_equal(tile_min, ref.stage("tile_min"))
    assert np.array_equal(tile_max, ref.stage("tile_max"))
    assert np.array_equal(state[STATE_SPAN], ref.stage("span_hist"))
    assert np.array_equal(state[STATE_MEAN], ref.stage("mean_hist"))
    assert np.array_equal(state[STATE_REF], ref.stage("ref")[:2])


def check_frame(img, family=0, gcfg=None, ocfg=None, stages=True):
    """GPU single-frame detect equals the oracle at every stage."""
    h, w = img.shape
    det = bdcudatag.Detector(family, w, h, gcfg)
    n, got = det.detect(img)
    ref = oracle.Frame(img, family, ocfg)
    wn, want = ref.detections()
    assert n == wn
    same_records(got, want)
    if stages:
        check_tile_stats(det.stage("tile_min"), det.stage("tile_max"), det.stage("state"), ref)
        rc = det.stage("row_count")
        assert np.array_equal(rc, ref.stage("row_count"))
        assert np.array_equal(det.stage("bits"), ref.stage("bits"))
        valid = np.zeros((h, ref.row_cap), bool)
        valid[np.arange(ref.row_cap)[None, :] < rc[:, None]] = True
        valid = valid.ravel()
        assert np.array_equal(det.stage("runs")[valid], ref.stage("runs")[valid])
        lab = det.stage("label")[valid]
        assert np.array_equal(lab, ref.stage("label")[valid])
        roots = np.unique(lab)
        assert np.array_equal(det.stage("area")[roots], ref.stage("area")[roots])
        assert np.array_equal(det.stage("bbox").reshape(-1, 4)[roots], ref.stage("bbox").reshape(-1, 4)[roots])
        nc = ref.candidate_count
        assert np.array_equal(det.stage("candidates")[:nc], ref.stage("candidates"))
        hq = det.stage("hull_quads")[:nc * 8]
        assert np.array_equal(hq.view(np.uint32), ref.stage("hull_quads")[:nc * 8].view(np.uint32))
        q = det.stage("quads")[family * ref.max_candidates * 8:][:nc * 8]
        assert np.array_equal(q.view(np.uint32), ref.stage("quads")[:nc * 8].view(np.uint32))
        dg = det.stage("decodes")[family * ref.max_candidates:][:nc]
        do = ref.stage("decodes")
        assert np.array_equal(dg["id"], do["id"])
        ok = do["id"] >= 0
        assert np.array_equal(dg[ok].view(np.uint8), do[ok].view(np.uint8))
    st = det.stats()
    c = ref.counts()
    assert st.runs == c[2] and st.quads == c[3] and st.detections == wn
    assert st.candidates == min(c[0], ref.max_candidates)
    assert st.roi_rows == min(c[4] * 8, h)
    return n, got
