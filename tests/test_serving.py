"""The serving loop (spatial_cell_gb300/serving.py): requests served
together give each request the same frame as serving it alone, and every
request finishes after its horizon."""
import pytest

from spatial_cell_gb300 import serving

pytestmark = pytest.mark.gpu


def test_results_equal_alone_and_in_the_mix(product):
    reqs = [serving.Request(0, 0.0, 101, 3000, 4, (0.5, 0.3, 0.1, 0.1)),
            serving.Request(1, 0.0, 102, 5000, 6, (0.2, 0.4, 0.2, 0.2)),
            serving.Request(2, 0.01, 103, 4096, 3, (0.25, 0.25, 0.25, 0.25))]
    res = serving.Server(budget_bytes=1 << 40).run(reqs)
    assert sorted(r.rid for r in res) == [0, 1, 2]
    for r in res:
        req = reqs[r.rid]
        assert r.steps == req.horizon and r.finished >= r.admitted >= req.arrival
        alone = serving.serve_alone(req)
        assert r.frame[0].tobytes() == alone[0].tobytes()
        assert r.frame[1].tobytes() == alone[1].tobytes()


def test_budget_admits_in_order(product):
    reqs = [serving.Request(k, 0.0, 200 + k, 3000, 2) for k in range(3)]
    one = reqs[0].bytes
    res = serving.Server(budget_bytes=one).run(reqs)   # room for one request at a time
    order = sorted(res, key=lambda r: r.admitted)
    assert [r.rid for r in order] == [0, 1, 2]
    for a, b in zip(order, order[1:]):
        assert b.admitted >= a.finished
