"""Static checks of the encounter task kernel's schedule constants
(merc_kernels.cuh): the hand-out order puts every (row, evaluation) unit
after the unit it depends on, the task decode covers every (unit, body,
part) exactly once, and the part-sum slots of a body do not overlap.  The
decode below restates the kernel's integer arithmetic from the constants
read out of the header."""
import os
import re

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "p9-integrator_gb300", "csrc",
                   "merc_kernels.cuh")


def _constants():
    src = open(HDR).read()
    m = re.search(r"constexpr unsigned kEncPartsBySlot = ([^;]+);", src)
    parts = re.findall(r"(\d+)u(?: << (\d+))?", m.group(1))
    p = [0] * 7  # parts per evaluation slot
    for v, shift in parts:
        p[int(shift or 0) // 4] = int(v)
    m = re.search(r"constexpr unsigned kEncOrder = ([^;]+);", src)
    units = re.findall(r"enc_unit\((\d), (\d)\)(?: << (\d+))?", m.group(1))
    order = [None] * len(units)
    for row, e, shift in units:
        order[int(shift or 0) // 4] = (int(row), int(e))
    return p, order


def _qoff(p, slot):
    return 3 * sum(p[:slot])


def _slot(row, e):
    return e if row == 2 else (4 + e if row == 1 else 6)


def test_order_respects_dependencies():
    p, order = _constants()
    assert sorted(order) == sorted([(2, 0), (2, 1), (2, 2), (2, 3), (1, 0), (1, 1), (0, 0)])
    for k, (row, e) in enumerate(order):
        if e > 0:
            assert order.index((row, e - 1)) < k, (row, e)
    assert order[0] == (2, 0), "the critical row starts first"


def test_decode_covers_every_task_once():
    p, order = _constants()
    for count in (1, 2, 7, 190):
        total = sum(p) * count
        seen = set()
        for t in range(total):
            unit, u = 0, t
            while u >= p[_slot(*order[unit])] * count:
                u -= p[_slot(*order[unit])] * count
                unit += 1
            row, e = order[unit]
            P = p[_slot(row, e)]
            k, q = divmod(u, P)
            assert 0 <= k < count and 0 <= q < P
            seen.add((row, e, k, q))
        assert len(seen) == total


def test_part_slots_do_not_overlap():
    p, _ = _constants()
    spans = []
    for row, evals in ((2, 4), (1, 2), (0, 1)):
        for e in range(evals):
            off = _qoff(p, _slot(row, e))
            spans.append((off, off + 3 * p[_slot(row, e)]))
    spans.sort()
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert a1 <= b0
    assert spans[0][0] == 0
    assert spans[-1][1] == 3 * sum(p)  # kEncQ
    assert all(1 <= v <= 15 for v in p)
