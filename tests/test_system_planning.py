"""Host-side planning of OpticalSystem, without a GPU: OpticalSequence expansion per
direction (optical_sequence.jl:54-70), PadCropOperator spans (pairing, nesting, the
direction swap, errors; pad_crop_operators.jl:291-356) and TiltAnchor's stored tilts.
The components here are stubs that only carry a name; nothing is launched."""

import numpy as np
import pytest

from __graft_entry__ import load_package


@pytest.fixture(scope="module")
def fo():
    return load_package()


class Grid:
    """The attributes of a ScalarField that planning reads."""

    def __init__(self, nx, ny, batch_shape=(), tilts=(0.0, 0.0)):
        self.nx, self.ny = nx, ny
        self.julia_batch_shape = batch_shape
        self.batch = int(np.prod(batch_shape)) if batch_shape else 1
        self.tilts = tilts

    def lambdas_per_field(self):
        return np.ones(self.batch)

    def tilts_per_field(self):
        from fluxoptics_gb300.fields import per_field
        tx = per_field(self.tilts[0], self.julia_batch_shape)
        ty = per_field(self.tilts[1], self.julia_batch_shape)
        return np.stack([np.broadcast_to(tx, (self.batch,)), np.broadcast_to(ty, (self.batch,))], axis=1)


def stubs(fo, *names):
    class Stub(fo.Component):
        def __init__(self, name):
            self.name = name

        def __repr__(self):
            return self.name

    return [Stub(n) for n in names]


def names(segs):
    out = []
    for s in segs:
        if type(s).__name__ == "_PaddedSpan":
            out.append(("span", names(s.inner.segments(Grid(64, 64)))))
        else:
            out.append(repr(s))
    return out


def test_sequence_order_per_direction(fo):
    a, b, c, d = stubs(fo, "a", "b", "c", "d")
    inner = fo.OpticalSequence(b, c)
    seq = fo.OpticalSequence(a, inner, d)
    assert fo.get_sequence(seq) == (a, inner, d)
    assert seq.expanded(fo.Forward) == [a, b, c, d]
    assert seq.expanded(fo.Backward) == [d, c, b, a]
    u = Grid(32, 32)
    fwd = fo.OpticalSystem(None, [seq, a], direction=fo.Forward)
    bwd = fo.OpticalSystem(None, [seq, a], direction=fo.Backward)
    assert fwd.leaf_components() == [a, b, c, d, a]
    # the system runs its own list in order; a sequence inside it runs reversed
    assert bwd.leaf_components() == [d, c, b, a, a]
    assert names(fwd.segments(u)) == ["a", "b", "c", "d", "a"]
    assert fo.get_components(fwd) == [seq, a]
    # FourierWrapper is a sequence: FFT, the components, inverse FFT
    fw = fo.FourierWrapper(u, b)
    parts = fw.expanded(fo.Backward)
    assert parts[1] is b and type(parts[0]).__name__ == "FourierOperator" and not parts[0].direct


def test_padded_spans(fo):
    u = Grid(48, 40)
    op = fo.PadCropOperator(u, (64, 64), offset=(8, 12))
    assert (op.n, op.p, op.offset) == ((48, 40), (64, 64), (8, 12))
    assert op.pads(fo.Forward) and not op.pads(fo.Backward)
    cr = fo.adjoint(op)
    assert not cr.pads(fo.Forward) and cr.pads(fo.Backward) and op.pairs_with(cr)
    a, b, c = stubs(fo, "a", "b", "c")
    s = fo.OpticalSystem(None, [a, op, b, c, cr, a])
    segs = s.segments(u)
    assert names(segs) == ["a", ("span", ["b", "c"]), "a"]
    assert s.segments(u)[1] is segs[1]  # the span is built once
    # nesting: a second pad inside the first span
    op2 = fo.PadCropOperator(Grid(64, 64), (128, 128))
    s2 = fo.OpticalSystem(None, [op, b, op2, c, fo.adjoint(op2), cr])
    seg = s2.segments(u)
    assert len(seg) == 1
    assert names(seg[0].inner.segments(Grid(64, 64))) == ["b", ("span", ["c"])]
    # Backward: the adjoint operator pads and the operator crops
    sb = fo.OpticalSystem(None, [cr, b, op], direction=fo.Backward)
    assert names(sb.segments(u)) == [("span", ["b"])]
    # a sequence holding a span stays a span in the Backward direction: reversed, the
    # adjoint operator comes first and pads there, and the operator crops
    seq = fo.OpticalSequence(op, b, cr)
    sq = fo.OpticalSystem(None, [seq], direction=fo.Backward)
    assert names(sq.segments(u)) == [("span", ["b"])]


def test_padded_span_errors(fo):
    u = Grid(48, 40)
    op = fo.PadCropOperator(u, (64, 64))
    a, = stubs(fo, "a")
    with pytest.raises(ValueError, match="no cropping partner"):
        fo.OpticalSystem(None, [op, a]).segments(u)
    with pytest.raises(ValueError, match="without a padding one"):
        fo.OpticalSystem(None, [fo.adjoint(op), a]).segments(u)
    other = fo.PadCropOperator(u, (64, 64), offset=(1, 0))
    with pytest.raises(ValueError, match="undoes its pad"):
        fo.OpticalSystem(None, [op, a, fo.adjoint(other)]).segments(u)
    with pytest.raises(ValueError, match="does not fit"):
        fo.PadCropOperator(u, (40, 64))
    with pytest.raises(ValueError):
        fo.PadCropOperator(u, (64, 64), offset=(-1, 0))
    with pytest.raises(TypeError):
        op.propagate_(u)


def test_tilt_anchor_stores_the_template_tilts(fo):
    u = Grid(16, 16, batch_shape=(3, 2), tilts=(0.01, np.array([0.0, 0.02, -0.03])))
    anc = fo.TiltAnchor(u)
    assert anc.params() == {} and not anc.trainable
    assert anc.tilts[0].shape == (3, 2) and np.allclose(anc.tilts[0], 0.01)
    assert np.allclose(anc.tilts[1][:, 0], [0.0, 0.02, -0.03]) and np.allclose(anc.tilts[1][:, 1], [0.0, 0.02, -0.03])
    single = fo.TiltAnchor(Grid(16, 16, tilts=(0.005, -0.002)))
    assert single.tilts == (0.005, -0.002)


def test_per_field_broadcast_follows_parse_val(fo):
    """Per-field wavelengths / tilts (src/Fields.jl:18-38): the value array keeps its own
    shape on the trailing dims (copyto! into a (1, 1, size(val)...) array) and broadcasts
    against the field; fields are listed in column-major order of the trailing dims."""
    from fluxoptics_gb300.fields import per_field
    assert np.array_equal(per_field(0.64, (3, 2)), np.full(6, 0.64))
    assert np.array_equal(per_field([1.0, 2.0, 3.0], (3, 2)), [1, 2, 3, 1, 2, 3])
    v = np.array([[1.0, 4.0], [2.0, 5.0], [3.0, 6.0]])  # Julia (3, 2): v[i, j] for field (i, j)
    assert np.array_equal(per_field(v, (3, 2)), [1, 2, 3, 4, 5, 6])
    assert np.array_equal(per_field([7.0], (3, 2)), np.full(6, 7.0))
    assert np.array_equal(per_field(np.array([[1.0, 2.0]]), (3, 2)), [1, 1, 1, 2, 2, 2])  # (1, 2) over d4
    assert np.array_equal(per_field([0.5], ()), [0.5])
    with pytest.raises(ValueError):
        per_field([1.0, 2.0], ())
    with pytest.raises(ValueError):
        per_field([1.0, 2.0], (3,))
