"""The per-item steps of the streaming FP32 step exist twice: written out in the
single-case kernel k_stream32 (fp32_stream.cu, where the shared inlined function
measured slower) and as stream_item (fp32_stream.cuh) for the batched serving kernel.
They must stay the same steps: the only differences allowed are where the segment's
rows come from, how the tensor map is passed and how a timed-out load ends the warp."""
import difflib
from pathlib import Path

CSRC = Path(__file__).resolve().parents[1] / 'mpdugks_gb300' / 'csrc'
START = "// the strip's window is columns hs .. hs+31"
END = "cp_async_wait_all();  // nothing in flight into this warp's buffers"


def body(text: str, indent: int) -> list[str]:
    a = text.index(START)
    a = text.rindex('\n', 0, a) + 1
    b = text.index(END, a)
    b = text.rindex('\n', 0, b) + 1
    return [ln[indent:] if ln.startswith(' ' * indent) else ln for ln in text[a:b].splitlines()]


def test_the_two_copies_of_the_item_steps_agree():
    kernel = body((CSRC / 'fp32_stream.cu').read_text(), 8)
    shared = body((CSRC / 'fp32_stream.cuh').read_text(), 4)
    diff = [ln for ln in difflib.unified_diff(kernel, shared, lineterm='', n=0)
            if ln.startswith(('-', '+')) and not ln.startswith(('---', '+++'))]
    allowed = {
        '-const int y0 = seg * seg_rows, y1 = min(y0 + seg_rows, ny);',
        '-                tma_load_row(smem_u32(stg + m4(j) * STG_SLOT), &tmap, hs, row_of(j), zin, bar);',
        '+                tma_load_row(smem_u32(stg + m4(j) * STG_SLOT), tmap_p, hs, row_of(j), zin, bar);',
        '-                return;',
        '+                return false;',
    }
    assert set(diff) <= allowed, '\n'.join(x for x in diff if x not in allowed)
