"""The prepared DOP853 batch's output arena (propagate.Dop853Batch): every
output part is an 8-byte aligned, non-overlapping view of one byte buffer,
and the result fields view the parts they name, so one copy of the buffer
moves every output.  Checked on CPU buffers with the batch's own layout and
carving code (no device work)."""
import pytest
import torch

from hiten_gb300 import propagate as P


def _views(n, dim, max_hits):
    b = P.Dop853Batch.__new__(P.Dop853Batch)  # the layout code only: no device buffers
    b.n, b.dim, b.mh = n, dim, max_hits
    b.layout = P.Dop853Batch.arena_layout(dim, n, max_hits)
    nbytes = sum(P.Dop853Batch.part_bytes(dt, s) for _, dt, s in b.layout)
    buf = torch.zeros(nbytes, dtype=torch.uint8)
    return b, buf, b._carve(buf)


@pytest.mark.parametrize("n,dim,max_hits", [(5, 6, 2), (16384, 6, 1), (7, 42, 0), (3, 6, 8)])
def test_parts_are_aligned_and_disjoint(n, dim, max_hits):
    b, buf, v = _views(n, dim, max_hits)
    spans = []
    for name, dt, shape in b.layout:
        t = v[name]
        assert tuple(t.shape) == shape and t.dtype == dt
        start = t.storage_offset() * t.element_size()
        assert start % 8 == 0
        spans.append((start, start + t.numel() * t.element_size()))
    spans.sort()
    assert all(a[1] <= b_[0] for a, b_ in zip(spans, spans[1:]))
    assert spans[-1][1] <= buf.numel()


def test_result_fields_view_their_parts():
    b, buf, v = _views(5, 6, 2)
    v["y_end"].copy_(torch.arange(30, dtype=torch.float64).view(6, 5))
    v["t_end"].fill_(-1.0)
    v["hits"][:10].fill_(2.0)
    v["hits"][10:].copy_(torch.arange(60, dtype=torch.float64))
    v["n_acc"].fill_(3)
    v["n_hits"].fill_(7)
    r = b._result(v)
    assert r.y_end.shape == (5, 6) and float(r.y_end[4, 5]) == 29.0 and float(r.y_end[1, 0]) == 1.0
    assert float(r.t_end[2]) == -1.0 and int(r.n_accept[0]) == 3 and int(r.n_hits[4]) == 7
    assert r.hit_t.shape == (5, 2) and float(r.hit_t[3, 1]) == 2.0
    # hit_y[i, k, c] is hits[10 + (k * 6 + c) * 5 + i]
    assert r.hit_y.shape == (5, 2, 6) and float(r.hit_y[4, 1, 5]) == (1 * 6 + 5) * 5 + 4
