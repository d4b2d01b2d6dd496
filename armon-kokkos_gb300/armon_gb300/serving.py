"""Replay of a request trace through the server (armon_server_*), in real time.

Request k is submitted once the wall clock since the start reaches its arrival time; between
arrivals the server runs rounds (admission, a few cycles of every running solve, retirement).
Time-to-solution is measured from the request's arrival to the end of the round that saw its loop
end (its final state is then on the device, ready to download).
"""
from __future__ import annotations

import time
from dataclasses import dataclass

from . import REQ_DONE, RequestInfo, Server
from .workloads import Request


@dataclass
class Served:
    index: int             # position in the trace
    arrival: float         # seconds after the start
    admitted: float        # seconds after the start (-1: never)
    done: float            # seconds after the start
    status: int
    precision: int
    cells: int
    cycles: int

    @property
    def tts(self) -> float:
        return self.done - self.arrival


def replay(server: Server, trace: list[Request], on_done=None, release: bool = True,
           time_limit: float | None = None) -> tuple[list[Served], float]:
    """Runs the trace to completion (or until time_limit seconds, after which no more requests are
    submitted and the ones submitted are finished).  on_done(req_id, index, info) is called for each
    finished request before it is released.  Returns the records in trace order and the wall time
    from the start to the last completion."""
    t0 = time.perf_counter()
    srv0 = None                 # server clock at t0 (its t_* are seconds since its creation)
    ids: dict[int, int] = {}
    out: dict[int, Served] = {}
    nxt = 0
    n = len(trace)
    last_done = 0.0
    while True:
        now = time.perf_counter() - t0
        while nxt < n and trace[nxt].arrival <= now and (time_limit is None or trace[nxt].arrival <= time_limit):
            spec = trace[nxt].spec
            rid = server.submit(spec.params(), spec.precision, spec.sod_interface())
            if srv0 is None:
                srv0 = server.info(rid).t_submit - (time.perf_counter() - t0)
            ids[rid] = nxt
            nxt += 1
        submitted_all = nxt >= n or (time_limit is not None and now > time_limit)
        running, queued = server.step()
        while (rid := server.next_done()) is not None:
            info: RequestInfo = server.info(rid)
            k = ids[rid]
            spec = trace[k].spec
            done = info.t_done - srv0
            out[k] = Served(index=k, arrival=trace[k].arrival, admitted=(info.t_admit - srv0) if info.t_admit >= 0 else -1,
                            done=done, status=info.status, precision=info.precision, cells=spec.nx * spec.ny,
                            cycles=info.cycle if info.status == REQ_DONE else 0)
            last_done = max(last_done, done)
            if on_done is not None:
                on_done(rid, k, info)
            if release:
                server.release(rid)
        if submitted_all and running == 0 and queued == 0 and len(out) == len(ids):
            break
        if running == 0 and queued == 0 and nxt < n:
            # idle until the next arrival
            wait = trace[nxt].arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.05))
    return [out[k] for k in sorted(out)], last_done


def percentile(xs: list[float], q: float) -> float:
    if not xs:
        return float("nan")
    s = sorted(xs)
    k = (len(s) - 1) * q
    lo = int(k)
    hi = min(lo + 1, len(s) - 1)
    return s[lo] + (s[hi] - s[lo]) * (k - lo)
