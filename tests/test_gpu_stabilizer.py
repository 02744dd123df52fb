"""The stabilizer tableau on the GPU against the oracle's restatement of
StabilizerBackend (src/backend/stabilizer.rs): identical generators (x, z
bits and signs) and classical registers for random Clifford circuits with
measurements and classical control, the reference's own tests re-expressed,
and the statevector cross-check of tests/stabilizer.rs (every generator has
expectation +1 on the GPU statevector)."""
import math

import numpy as np
import pytest

import oracle as O
from everett_gb300 import Circuit, CudaStateVectorBackend, Gate1, Gate2, Rng
from everett_gb300.circuit import Apply1
from everett_gb300.error import NonClifford
from everett_gb300.stabilizer import StabilizerBackend

pytestmark = pytest.mark.gpu


def random_clifford(rng: Rng, n: int, depth: int, measure: bool) -> Circuit:
    c = Circuit.with_classical(n, n) if measure else Circuit(n)
    one = [lambda q: c.h(q), lambda q: c.s(q), lambda q: c.x(q), lambda q: c.y(q),
           lambda q: c.z(q), lambda q: c.gate1(Gate1.s().adjoint(), q),
           lambda q: c.rz(q, math.pi / 2), lambda q: c.rz(q, math.pi), lambda q: c.gate1(Gate1.id(), q)]
    for _ in range(depth):
        k = int(rng.next_u64() % 12)
        a = int(rng.next_u64() % n)
        b = int(rng.next_u64() % n)
        if n > 1 and b == a:
            b = (a + 1) % n
        if k < 9 or n == 1:
            one[k % 9](a)
        elif k == 9:
            c.cnot(a, b)
        elif k == 10:
            c.gate2([Gate2.cz(), Gate2.swap(), Gate2.cnot()][int(rng.next_u64() % 3)], a, b)
        else:
            c.controlled([b], [Gate1.x(), Gate1.z()][int(rng.next_u64() % 2)], a)
        if measure and rng.next_u64() % 7 == 0:
            q = int(rng.next_u64() % n)
            c.measure(q, q)
            if rng.next_u64() % 2:
                c.if_classic(q, Apply1(Gate1.h(), int(rng.next_u64() % n)))
    return c


def test_random_clifford_circuits_match_oracle(gpu):
    rng = Rng.seed_from_u64(0xC11FF)
    for case in range(60):
        n = [1, 2, 3, 5, 8, 31, 64, 65, 100, 130][case % 10]
        c = random_clifford(rng, n, 4 * n + 10, measure=case % 2 == 1)
        for seed in (0, case):
            want = O.stab_run(c, seed)
            ex = StabilizerBackend.run_seeded(c, seed)
            x, z, neg, bits = want
            assert ex.classical() == bits, (case, n, seed)
            for i, g in enumerate(ex.generators()):
                assert np.array_equal(g.x, x[i].astype(bool)), (case, i)
                assert np.array_equal(g.z, z[i].astype(bool)), (case, i)
                assert g.neg == bool(neg[i]), (case, i)


def test_reference_assertions(gpu):
    """backend/stabilizer.rs tests: GHZ has n generators; T and rx(0.3) are
    rejected; rz(pi/2) is accepted as S; Bell halves agree for 32 seeds;
    |0> measures 0; a 200-qubit GHZ is feasible."""
    c = Circuit(4)
    c.h(0).cnot(0, 1).cnot(1, 2).cnot(2, 3)
    assert len(StabilizerBackend.run(c).generators()) == 4
    for bad in (lambda k: k.t(0), lambda k: k.rx(0, 0.3)):
        k = Circuit(1)
        bad(k)
        with pytest.raises(NonClifford) as e:
            StabilizerBackend.run(k)
        assert "Clifford" in str(e.value)
    k = Circuit(1)
    k.rz(0, math.pi / 2)
    StabilizerBackend.run(k)
    for seed in range(32):
        b = Circuit.with_classical(2, 2)
        b.h(0).cnot(0, 1).measure(0, 0).measure(1, 1)
        cl = StabilizerBackend.run_seeded(b, seed).classical()
        assert cl[0] == cl[1]
    z = Circuit.with_classical(1, 1)
    z.measure(0, 0)
    assert StabilizerBackend.run(z).classical() == [False]
    g = Circuit(200)
    g.h(0)
    for q in range(199):
        g.cnot(q, q + 1)
    assert len(StabilizerBackend.run(g).generators()) == 200
    # a multi-controlled gate and a controlled non-Pauli are not Clifford
    k = Circuit(3)
    k.controlled([0, 1], Gate1.x(), 2)
    with pytest.raises(NonClifford):
        StabilizerBackend.run(k)


def test_generators_stabilize_the_statevector(gpu):
    """tests/stabilizer.rs: every generator has expectation +1 on the
    statevector of the same circuit."""
    rng = Rng.seed_from_u64(0x5EED)
    for case in range(30):
        n = 2 + case % 7
        c = random_clifford(rng, n, 25, measure=False)
        gens = StabilizerBackend.run(c).generators()
        assert len(gens) == n
        st = CudaStateVectorBackend.run(c).state()
        vals = st.pauli_expectation(gens)
        assert np.max(np.abs(vals - 1.0)) < 1e-9, (case, [str(g) for g in gens], vals)
