"""Balanced work units of the TMA column pass (host code in csrc/fo_units.h, built
here with g++): every (strip, field) is covered exactly once, full units keep the
2-D launch order, and a partly filled last round is spread over the slots."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dump(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ is not available")
    exe = str(tmp_path_factory.mktemp("units") / "col_units_dump")
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "fluxoptics.jl_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "col_units_dump.cpp"), "-o", exe], check=True)

    def run(items, strips, slots):
        out = subprocess.run([exe, str(strips), str(slots), *map(str, items)], check=True,
                             capture_output=True, text=True).stdout
        return [tuple(map(int, ln.split())) for ln in out.splitlines()]
    return run


def items_of(batch, per_item, per_table):
    """Runs of at most per_item fields that do not cross a table boundary."""
    offs = [0]
    for i in range(1, batch + 1):
        if i == batch or i % per_table == 0 or i - offs[-1] >= per_item:
            offs.append(i)
    return offs


@pytest.mark.parametrize("batch,per_table,strips,slots", [
    (48, 16, 512, 152),    # the 2048^2 x 48 headline: 1536 blocks, last round of 16
    (16, 16, 512, 152),    # 16 fields: 512 blocks, last round of 56
    (48, 16, 1024, 304),   # 2-column strips at two CTAs per SM
    (7, 7, 128, 152),      # fits in one round: no units
    (45, 15, 512, 152),    # 3 x 15 fields
    (3, 1, 256, 152),      # single-field items cannot be cut
])
def test_units_cover_every_field_strip_once(dump, batch, per_table, strips, slots):
    items = items_of(batch, 16, per_table)
    n_items = len(items) - 1
    units = dump(items, strips, slots)
    total = n_items * strips
    if total <= slots:
        assert units == []
        return
    seen = set()
    for first, end, strip in units:
        assert 0 <= strip < strips and first < end
        assert any(items[i] <= first and end <= items[i + 1] for i in range(n_items))  # within one item
        for f in range(first, end):
            assert (strip, f) not in seen
            seen.add((strip, f))
    assert len(seen) == batch * strips
    # the full rounds keep the 2-D launch order; only the last partial round is cut
    full = total - total % slots
    blocks = [(items[i], items[i + 1], st) for st in range(strips) for i in range(n_items)]
    assert units[:full] == blocks[:full]
    tail = total % slots
    if tail and min(items[i + 1] - items[i] for i in range(n_items)) > 1:
        assert len(units) - full > tail          # the last round was spread
        assert len(units) - full <= max(slots, tail)


def test_empty_items_make_no_units(dump):
    """An empty run of fields (equal offsets) must not become a unit: the
    persistent column kernel loads the next unit's first strip from inside the
    current unit's field loop, so a unit without fields would leave that load
    unissued."""
    items = [0, 16, 16, 32, 48, 48]  # two empty items among three full ones
    strips, slots = 512, 152
    units = dump(items, strips, slots)
    assert units, "1536 non-empty blocks need units"
    seen = set()
    for first, end, strip in units:
        assert first < end
        for f in range(first, end):
            assert (strip, f) not in seen
            seen.add((strip, f))
    assert len(seen) == 48 * strips
