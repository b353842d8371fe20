"""Host logic of the serving loop (serve.Server) against a stand-in batch on
the CPU: backfilled admission (a request that does not fit is passed over,
later ones that fit start), the age cap (an old request keeps its place until
it fits), asynchronous ticks (updates queued before admission, waited for
after it), and the bookkeeping of finished requests."""
import hydrocuda
import serve


class FakeBatch:
    """Budget in cells; an instance finishes after `need` updates (its tag % 7 + 3)."""

    def __init__(self, budget_cells):
        self.budget = budget_cells
        self.used = 0
        self.slot_desc = {}
        self.live = {}          # slot -> [tag, cells, steps, need]
        self.next_slot = 0
        self.queued = 0
        self.calls = []

    def _admit(self, args, tag):
        cells = 1
        for n in args["gridSize"]:
            cells *= n
        if self.used + cells > self.budget:
            return None
        slot = self.next_slot
        self.next_slot += 1
        self.used += cells
        self.slot_desc[slot] = hydrocuda.make_desc(args)
        self.live[slot] = [tag, cells, 0, tag % 7 + 3]
        self.calls.append(("admit", tag))
        return slot

    def try_admit(self, args, cons, t_end, tag=0, layout="aos6"):
        return self._admit(args, tag)

    def try_admit_init(self, args, kind, t_end, tag=0, **params):
        return self._admit(args, tag)

    def _advance(self, k):
        for v in self.live.values():
            v[2] = min(v[2] + k, v[3])

    def step_async(self, k):
        self.calls.append(("step_async", k))
        self.queued += k

    def wait(self):
        self.calls.append(("wait",))
        self._advance(self.queued)
        self.queued = 0

    def step(self, k):
        self._advance(k)

    def poll(self):
        out = []
        for slot, (tag, cells, steps, need) in self.live.items():
            if steps >= need and not getattr(self, "_rep_%d" % slot, False):
                setattr(self, "_rep_%d" % slot, True)
                out.append(dict(slot=slot, tag=tag, steps=steps, t=0.1, status=0))
        return out

    def fetch(self, slot, layout="aos6"):
        return None

    def retire(self, slot):
        tag, cells, steps, need = self.live.pop(slot)
        self.used -= cells


def _req(tag, arrival, n):
    args = dict(dim=2, gridSize=[n, n], mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
                usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2", cfl=.3)
    return serve.Request(arrival, args, None, 0.1, tag, init=("sod", {}))


def _clock():
    t = [0.0]

    def clock():
        t[0] += 1e-3
        return t[0]
    return clock


def test_backfill_admits_smaller_requests_past_one_that_does_not_fit():
    b = FakeBatch(budget_cells=100 * 100)
    reqs = [_req(0, 0.0, 80), _req(1, 0.0, 90), _req(2, 0.0, 20), _req(3, 0.0, 30)]
    srv = serve.Server(b, steps_per_tick=1, keep_results=False, age_cap_s=1e9)
    done = srv.run(reqs, clock=_clock(), sleep=lambda s: None)
    assert sorted(r.tag for r in done) == [0, 1, 2, 3]
    admits = [c[1] for c in b.calls if c[0] == "admit"]
    # request 1 (90^2) does not fit beside request 0 (80^2): 2 and 3 start before it
    assert admits.index(2) < admits.index(1) and admits.index(3) < admits.index(1)
    assert srv.passed_over >= 2


def test_age_cap_keeps_an_old_request_first():
    b = FakeBatch(budget_cells=100 * 100)
    reqs = [_req(0, 0.0, 80), _req(1, 0.0, 90), _req(2, 0.0, 20), _req(3, 0.0, 30)]
    srv = serve.Server(b, steps_per_tick=1, keep_results=False, age_cap_s=0.0)
    srv.run(reqs, clock=_clock(), sleep=lambda s: None)
    admits = [c[1] for c in b.calls if c[0] == "admit"]
    # with no patience, nothing goes ahead of the oldest waiting request
    assert admits == [0, 1, 2, 3]
    assert srv.passed_over == 0


def test_ticks_are_queued_before_admission_and_waited_after():
    b = FakeBatch(budget_cells=10 ** 6)
    reqs = [_req(k, 0.002 * k, 10 + k) for k in range(12)]
    srv = serve.Server(b, steps_per_tick=2, keep_results=False)
    done = srv.run(reqs, clock=_clock(), sleep=lambda s: None)
    assert len(done) == 12
    assert srv.cell_updates == sum((r.tag % 7 + 3) * (10 + r.tag) ** 2 for r in done)
    # every wait closes a tick queued earlier in the same pass
    depth = 0
    for c in b.calls:
        if c[0] == "step_async":
            depth += 1
        elif c[0] == "wait":
            depth -= 1
            assert depth == 0
    assert any(b.calls[i][0] == "step_async" and b.calls[i + 1][0] == "admit" for i in range(len(b.calls) - 1))
