"""Host logic of the fused integrator: the stage plan with buffer reuse must
reproduce the reference's Runge-Kutta sequence (hydro/int/rk.lua:98-218).

The plan is read back through a small C++ probe compiled against the
library's planner source, and executed here on scalar states with a
nonlinear stand-in for L, once as the reference sequences it (fresh buffers,
alpha terms then beta terms, ascending k) and once through the plan's buffer
assignments."""
import os
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "hydro-cl-lua_gb300", "csrc")

PROBE = r"""
#include <cstdio>
#include "hc_internal.h"
namespace hc { void set_error(const std::string&) {} int fail(int c, const std::string&) { return c; }
int cuda_fail(cudaError_t, const char*) { return -2; } }
int main() {
    for (int integ = 0; integ < HC_NUM_INTEGRATORS; ++integ) {
        hc::IntegratorPlan P = hc::make_plan(integ);
        std::printf("I %d %d %d %d %d\n", integ, P.n_stages, P.n_state_bufs, P.n_deriv_bufs, P.result_buf);
        for (int s = 0; s < P.n_stages; ++s) {
            const hc::StagePlan& S = P.stage[s];
            std::printf("S %d %d %d %d %.17g %d %d", S.in_buf, S.out_buf, S.store_deriv, S.last, S.beta_cur, S.n_alpha, S.n_beta);
            for (int k = 0; k < S.n_alpha; ++k) std::printf(" %d %.17g", S.alpha[k].buf, S.alpha[k].coef);
            for (int k = 0; k < S.n_beta; ++k) std::printf(" %d %.17g", S.beta[k].buf, S.beta[k].coef);
            std::printf("\n");
        }
    }
}
"""


@pytest.fixture(scope="module")
def plans(tmp_path_factory):
    d = tmp_path_factory.mktemp("plan")
    src = d / "probe.cu"
    src.write_text(PROBE)
    exe = d / "probe"
    subprocess.check_call(["nvcc", "-std=c++17", "-I", CSRC, str(src), os.path.join(CSRC, "hc_plan.cu"), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split("\n")
    plans = {}
    cur = None
    for line in out:
        t = line.split()
        if not t:
            continue
        if t[0] == "I":
            cur = dict(n_stages=int(t[2]), n_state=int(t[3]), n_deriv=int(t[4]), result=int(t[5]), stages=[])
            plans[int(t[1])] = cur
        else:
            in_b, out_b, store, last = map(int, t[1:5])
            bc = float(t[5])
            na, nb = int(t[6]), int(t[7])
            rest = t[8:]
            alpha = [(int(rest[2 * k]), float(rest[2 * k + 1])) for k in range(na)]
            rest = rest[2 * na:]
            beta = [(int(rest[2 * k]), float(rest[2 * k + 1])) for k in range(nb)]
            cur["stages"].append(dict(inb=in_b, outb=out_b, store=store, last=last, bcur=bc, alpha=alpha, beta=beta))
    return plans


# alpha / beta tables of hydro/int/all.lua (forward Euler as a 1-stage table)
TABLES = {
    0: ([[1]], [[1]]),
    1: ([[1, 0], [1, 0]], [[.5, 0], [0, 1]]),
    2: ([[1, 0], [1, 0]], [[1, 0], [.5, .5]]),
    3: ([[1, 0], [1, 0]], [[2 / 3, 0], [1 / 4, 3 / 4]]),
    4: ([[1, 0, 0], [1, 0, 0], [1, 0, 0]], [[.5, 0, 0], [-1, 2, 0], [1 / 6, 2 / 6, 1 / 6]]),
    5: ([[1, 0, 0, 0]] * 4, [[.5, 0, 0, 0], [0, .5, 0, 0], [0, 0, 1, 0], [1 / 6, 2 / 6, 2 / 6, 1 / 6]]),
    6: ([[1, 0, 0, 0]] * 4, [[1 / 3, 0, 0, 0], [-1 / 3, 0, 0, 0], [1, -1, 1, 0], [1 / 8, 3 / 8, 3 / 8, 1 / 8]]),
    7: ([[1, 0], [.5, .5]], [[1, 0], [0, .5]]),
    8: ([[1, 0], [1, 0]], [[-20, 0], [41 / 40, -1 / 40]]),
    9: ([[1, 0, 0], [3 / 4, 1 / 4, 0], [1 / 3, 0, 2 / 3]], [[1, 0, 0], [0, 1 / 4, 0], [0, 0, 2 / 3]]),
    10: ([[1, 0, 0, 0], [649 / 1600, 951 / 1600, 0, 0], [53989 / 2500000, 4806213 / 20000000, 23619 / 32000, 0],
          [1 / 5, 6127 / 30000, 7873 / 30000, 1 / 3]],
         [[.5, 0, 0, 0], [-10890423 / 25193600, 5000 / 7873, 0, 0], [-102261 / 5000000, -5121 / 20000, 7873 / 10000, 0],
          [1 / 10, 1 / 6, 0, 1 / 6]]),
    11: ([[1, 0, 0, 0], [1, 0, 0, 0], [1, 0, 0, 0], [-1 / 3, 1 / 3, 2 / 3, 1 / 3]],
         [[.5, 0, 0, 0], [0, .5, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1 / 6]]),
}


def Lop(u):
    return np.sin(3 * u) - 0.5 * u * u


def reference_rk(alpha, beta, u0, dt):
    order = len(alpha)
    U = [None, u0]
    D = [None]
    for s in range(1, order + 1):
        D.append(Lop(U[s]))
        acc = np.zeros_like(u0)
        for k in range(1, s + 1):
            if alpha[s - 1][k - 1] != 0:
                acc = acc + U[k] * alpha[s - 1][k - 1]
        for k in range(1, s + 1):
            if beta[s - 1][k - 1] != 0:
                acc = acc + D[k] * (beta[s - 1][k - 1] * dt)
        U.append(acc)
    return U[-1]


def planned_rk(plan, u0, dt):
    bufs = {0: u0.copy()}
    dbufs = {}
    for S in plan["stages"]:
        src = bufs[S["inb"]]
        d = Lop(src)
        acc = np.zeros_like(u0)
        for b, c in S["alpha"]:
            acc = acc + bufs[b] * c
        for b, c in S["beta"]:
            acc = acc + dbufs[b] * (c * dt)
        if S["bcur"] != 0:
            acc = acc + d * (S["bcur"] * dt)
        if S["store"] >= 0:
            dbufs[S["store"]] = d
        assert S["outb"] != S["inb"]
        bufs[S["outb"]] = acc
    return bufs[plan["result"]]


@pytest.mark.parametrize("integ", range(12))
def test_plan_reproduces_reference_sequence(plans, integ):
    P = plans[integ]
    alpha, beta = TABLES[integ]
    assert P["n_stages"] == len(alpha)
    assert P["stages"][-1]["last"] == 1
    assert P["n_state"] <= 4 and P["n_deriv"] <= 4
    u0 = np.linspace(-1, 2, 17)
    np.testing.assert_array_equal(planned_rk(P, u0, 0.013), reference_rk(alpha, beta, u0, 0.013))


def test_state_stays_in_place_when_the_table_allows(plans):
    for integ in range(1, 12):
        assert plans[integ]["result"] == 0, oracle.INTEGRATORS[integ]
    assert plans[0]["result"] == 1   # forward Euler alternates between two buffers
