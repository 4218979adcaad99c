"""Per-frame metrics log (semantic_icpslam_gb300.metrics): JSON lines with
the frame stats and Mapping::CheckVisPercent's visible share."""
import io
import json

from semantic_icpslam_gb300 import _lib
from semantic_icpslam_gb300.metrics import FrameLog, visible_percent


def _stats(**kw):
    st = _lib.FrameStats()
    for k, v in kw.items():
        setattr(st, k, v)
    st.pose[0] = st.pose[5] = st.pose[10] = st.pose[15] = 1.0
    st.pose[3], st.pose[7], st.pose[11] = 0.5, -0.25, 1.0
    return st


def test_visible_percent_follows_check_vis_percent():
    # heapCounter counts the free blocks down: 1000 blocks, 400 left, 150 visible
    assert abs(visible_percent(_stats(visible=150, heap_counter=400), 1000) - 150 / 600) < 1e-12
    # an exhausted heap (counter below zero) counts as zero left
    assert abs(visible_percent(_stats(visible=10, heap_counter=-3), 100) - 0.1) < 1e-12


def test_frame_log_writes_one_line_per_frame(capsys):
    buf = io.StringIO()
    log = FrameLog(buf, 1000, echo=True)
    log.write(_stats(tracked=1, accepted=1, iterations=19, icp_error=1e-5, icp_count=250000, visible=300,
                     heap_counter=500))
    log.write(_stats(tracked=0, accepted=0, fail=1, state=0, missed=1))
    log.write(_stats(tracked=0, accepted=0, fail=2, icp_error=3e-4, missed=2), host_ms=0.5)
    lines = [json.loads(x) for x in buf.getvalue().splitlines()]
    assert [r["frame"] for r in lines] == [0, 1, 2]
    assert lines[0]["visible_percent"] == 300 / 500 and lines[0]["t"] == [0.5, -0.25, 1.0]
    assert [r["fail"] for r in lines] == ["ok", "icp_count_or_nan", "rejected"]
    assert lines[2]["host_ms"] == 0.5 and lines[2]["missed"] == 2
    out = capsys.readouterr().out.splitlines()
    assert out[0] == "track icp failed" and out[1].startswith("bad : ")
