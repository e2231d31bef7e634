"""State-vector application (sqg_apply_state, up to 30 qubits) against the oracle: fused
blocks and one pass per gate, batches, the drop-in Circuit.apply_to on 1-D states, and at
sizes the oracle cannot reach, size-independent properties (norm, fused == unfused, a circuit
followed by its adjoint giving the state back at 27 and 30 qubits)."""
import importlib

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def wl():
    return importlib.import_module("sequential-quantum-gate-decomposer_gb300.workloads")


def random_state(n, rng, batch=None):
    shape = (1 << n,) if batch is None else (batch, 1 << n)
    v = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


@pytest.mark.parametrize("n,gates", [(3, 40), (12, 300), (14, 400), (16, 300)])
def test_state_matches_oracle(sqg, wl, n, gates):
    rng = np.random.default_rng(100 + n)
    c = wl.all_gates_circuit(n, gates, rng)
    P = c.get_Parameter_Num()
    p = rng.uniform(0, 2 * np.pi, P)
    psi = random_state(n, rng)
    ref = O.apply_to(n, c.gate_records(), p, psi.reshape(-1, 1).copy()).reshape(-1)
    th = torch.from_numpy(p).cuda()
    for fused in (True, False):
        d = torch.from_numpy(psi.copy()).cuda()
        c.apply_state_device(th, d, fused=fused)
        torch.cuda.synchronize()
        assert float(np.abs(d.cpu().numpy() - ref).max()) < 1e-12, fused
    assert 1 <= c.state_block_count() <= c.get_Gate_Num()


def test_state_batch_and_dropin_apply_to(sqg, wl):
    n, B = 15, 3
    rng = np.random.default_rng(7)
    c = wl.all_gates_circuit(n, 200, rng)
    P = c.get_Parameter_Num()
    p = rng.uniform(0, 2 * np.pi, (B, P))
    psi = random_state(n, rng, B)
    d = torch.from_numpy(psi.copy()).cuda()
    c.apply_state_device(torch.from_numpy(p).cuda(), d)
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    for b in range(B):
        ref = O.apply_to(n, c.gate_records(), p[b], psi[b].reshape(-1, 1).copy()).reshape(-1)
        assert float(np.abs(got[b] - ref).max()) < 1e-12
    # Circuit.apply_to on a 1-D state works in place, as the reference's (qgd_Circuit.py:546)
    v = psi[0].copy()
    c.apply_to(p[0], v)
    assert float(np.abs(v - got[0]).max()) < 1e-13


def test_matrix_entry_points_reject_large_registers(sqg, wl):
    c = wl.all_gates_circuit(14, 10, np.random.default_rng(1))
    with pytest.raises(Exception):
        c.get_Matrix(np.zeros(c.get_Parameter_Num()))


@pytest.mark.parametrize("n", [20, 24])
def test_qc_sim_circuit_large_state(sqg, wl, n):
    """The reference's simulation-benchmark circuit at sizes beyond the oracle: the norm is
    kept to 1e-12 and fused blocks give the result of one pass per gate."""
    rng = np.random.default_rng(n)
    c = wl.qc_sim_circuit(n, levels=4 if n == 20 else 1)
    th = torch.from_numpy(rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())).cuda()
    psi = torch.from_numpy(random_state(n, rng)).cuda()
    a = psi.clone()
    b = psi.clone()
    c.apply_state_device(th, a, fused=True)
    c.apply_state_device(th, b, fused=False)
    torch.cuda.synchronize()
    assert abs(float(torch.linalg.vector_norm(a)) - 1.0) < 1e-12
    assert float((a - b).abs().max()) < 1e-12
    assert c.state_block_count() < c.get_Gate_Num() / 4


@pytest.mark.parametrize("n,gates,mq", [(14, 400, 4), (16, 300, 7), (12, 300, 3)])
def test_partitioned_circuit_state_matches_oracle(sqg, wl, n, gates, mq):
    """A Kahn-partitioned circuit (PartitionCircuit) applied with fused passes that break only
    at partition boundaries gives the original circuit's state."""
    part = importlib.import_module("sequential-quantum-gate-decomposer_gb300.partitioning")
    rng = np.random.default_rng(200 + n)
    c = wl.all_gates_circuit(n, gates, rng)
    p = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    pc, pp, parts = part.PartitionCircuit(c, p, mq)
    psi = random_state(n, rng)
    ref = O.apply_to(n, c.gate_records(), p, psi.reshape(-1, 1).copy()).reshape(-1)
    d = torch.from_numpy(psi.copy()).cuda()
    pc.apply_state_device(torch.from_numpy(pp).cuda(), d)
    torch.cuda.synchronize()
    assert float(np.abs(d.cpu().numpy() - ref).max()) < 1e-12
    assert 1 <= pc.state_block_count() <= len(parts)


def test_qasm_program_partitioned_and_simulated(sqg, wl):
    """The reference's simulation flow: an OpenQASM program, partitioned (Kahn), applied to a
    state with fused passes that break only at partition boundaries, against the oracle applying
    the unpartitioned program; and the partition hand-over rejects malformed boundaries."""
    qasm = importlib.import_module("sequential-quantum-gate-decomposer_gb300.qasm")
    lib = importlib.import_module("sequential-quantum-gate-decomposer_gb300._native")
    rng = np.random.default_rng(17)
    n = 13
    lines = ["OPENQASM 2.0;", 'include "qelib1.inc";', "qreg q[%d];" % n]
    for _ in range(300):
        a, b = (int(v) for v in rng.permutation(n)[:2])
        lines.append(["h q[%d];" % a, "cx q[%d],q[%d];" % (a, b), "rz(%r) q[%d];" % (float(rng.uniform(-3, 3)), a),
                      "cz q[%d],q[%d];" % (a, b), "u3(0.3,%r,0.1) q[%d];" % (float(rng.uniform(-3, 3)), a),
                      "cry(%r) q[%d],q[%d];" % (float(rng.uniform(-3, 3)), a, b)][rng.integers(6)])
    text = "\n".join(lines)
    circ, params, phase = qasm.qasm_to_circuit(text)
    assert phase == 0.0
    pc, pparams, parts = qasm.PartitionCircuitQasm(text, 5)
    psi = random_state(n, rng)
    ref = O.apply_to(n, circ.gate_records(), params, psi.reshape(-1, 1).copy()).reshape(-1)
    d = torch.from_numpy(psi.copy()).cuda()
    pc.apply_state_device(torch.from_numpy(pparams).cuda(), d)
    torch.cuda.synchronize()
    assert float(np.abs(d.cpu().numpy() - ref).max()) < 1e-12
    assert pc.state_block_count() <= len(parts)
    h = circ.native().handle
    L = circ.get_Gate_Num()
    for ends in ([L - 1], [5, 3, L], [L + 1]):
        arr = np.asarray(ends, dtype=np.int32)
        assert lib.lib().sqg_circuit_set_partitions(h, arr.ctypes.data, arr.size) == 1  # invalid argument
    arr = np.asarray([], dtype=np.int32)
    assert lib.lib().sqg_circuit_set_partitions(h, None, 0) == 0  # back to the gate-order plan


def test_second_renyi_entropy(sqg, wl):
    """Bell pair: S2 of one qubit is log 2; a product state has S2 = 0; against a direct numpy
    reduced density matrix of a random 10-qubit circuit's output."""
    c = sqg.Circuit(3)
    c.add_U3(0)            # H = U3(pi/2, 0, pi): stored (pi/4, 0, pi)
    c.add_CNOT(1, 0)
    c.add_adaptive(2, 1)   # a CRY at angle 0: the identity
    p = np.array([np.pi / 4, 0.0, np.pi, 0.0])
    assert np.isclose(c.get_Second_Renyi_Entropy(p, qubit_list=[0]), np.log(2), atol=1e-12)
    assert np.isclose(c.get_Second_Renyi_Entropy(p, qubit_list=[2]), 0.0, atol=1e-12)
    assert np.isclose(c.get_Second_Renyi_Entropy(p), 0.0, atol=1e-12)
    assert c.get_Second_Renyi_Entropy(None) is None
    rng = np.random.default_rng(33)
    n = 10
    c = wl.all_gates_circuit(n, 120, rng)
    th = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    psi = random_state(n, rng)
    out = O.apply_to(n, c.gate_records(), th, psi.reshape(-1, 1).copy()).reshape(-1)
    keep = [1, 4, 7, 8]
    t = out.reshape([2] * n).transpose([n - 1 - q for q in keep] + [n - 1 - q for q in range(n) if q not in keep])
    M = t.reshape(1 << len(keep), -1)
    rho = M @ M.conj().T
    want = -np.log(np.sum(np.abs(rho) ** 2))
    assert np.isclose(c.get_Second_Renyi_Entropy(th, psi, keep), want, atol=1e-10)


def _inverse(sqg, c, theta):
    """The adjoint circuit: gates in reverse order, each inverted through its parameters (U3
    with stored (t, p, l) -> (-t, -l, -p); RX, RY, RZ, CRY negated; CNOT, CZ their own inverse)."""
    inv = sqg.Circuit(c.qbit_num)
    recs = c.gate_records()
    params = []
    for t, tg, ctl, ps in recs[::-1]:
        t, tg, ctl, ps = int(t), int(tg), int(ctl), int(ps)
        if t == sqg.U3:
            inv.add_U3(tg)
            params += [-theta[ps], -theta[ps + 2], -theta[ps + 1]]
        elif t in (sqg.RX, sqg.RY, sqg.RZ):
            getattr(inv, {sqg.RX: "add_RX", sqg.RY: "add_RY", sqg.RZ: "add_RZ"}[t])(tg)
            params.append(-theta[ps])
        elif t == sqg.CRY:
            inv.add_CRY(tg, ctl)
            params.append(-theta[ps])
        else:
            getattr(inv, "add_CNOT" if t == sqg.CNOT else "add_CZ")(tg, ctl)
    return inv, np.asarray(params, dtype=np.float64)


@pytest.mark.parametrize("n", [27, 30])
def test_largest_registers_round_trip(sqg, wl, n):
    """At the largest registers (2^30 amplitudes, 16 GiB, the limit of sqg_apply_state) a
    circuit of every gate kind followed by its adjoint gives back the state, fused and one pass
    per gate, and the norm is kept: checks that index arithmetic holds up to the last qubit."""
    rng = np.random.default_rng(300 + n)
    c = wl.all_gates_circuit(n, 48, rng)
    for q in (n - 1, n - 2, 0):  # gates on the highest qubits for certain
        c.add_CRY(q, (q + 1) % n)
        c.add_U3(q)
    theta = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    inv, theta_inv = _inverse(sqg, c, theta)
    th = torch.from_numpy(theta).cuda()
    th_inv = torch.from_numpy(theta_inv).cuda()
    N = 1 << n
    psi = torch.empty(N, dtype=torch.complex128, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(n)
    psi.real.normal_(generator=gen)
    psi.imag.normal_(generator=gen)
    psi /= torch.linalg.vector_norm(psi)
    head = slice(0, 1 << 20)
    for fused in (True, False):
        v = psi.clone()
        c.apply_state_device(th, v, fused=fused)
        assert abs(float(torch.linalg.vector_norm(v)) - 1.0) < 1e-12
        assert float((v[head] - psi[head]).abs().max()) > 1e-6  # the circuit did act
        inv.apply_state_device(th_inv, v, fused=fused)
        v.sub_(psi)  # in place: at 30 qubits each full-size temporary is 16 GiB
        torch.cuda.synchronize()
        assert float(v.abs().max()) < 1e-12
        del v
        torch.cuda.empty_cache()
    del psi
    torch.cuda.empty_cache()


def test_largest_matrix_register_round_trip(sqg, wl):
    """13 qubits, the largest register of the matrix entry points (an 8192 x 8192 complex128
    target, 1 GiB): a circuit of every gate kind followed by its adjoint gives back the matrix,
    fused and one pass per gate."""
    n = 13
    rng = np.random.default_rng(313)
    c = wl.all_gates_circuit(n, 40, rng)
    c.add_CRY(n - 1, 0)
    c.add_U3(n - 1)
    theta = rng.uniform(0, 2 * np.pi, c.get_Parameter_Num())
    inv, theta_inv = _inverse(sqg, c, theta)
    th = torch.from_numpy(theta).cuda()
    th_inv = torch.from_numpy(theta_inv).cuda()
    N = 1 << n
    m = torch.empty((N, N), dtype=torch.complex128, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(n)
    m.real.normal_(generator=gen)
    m.imag.normal_(generator=gen)
    for fused in (True, False):
        v = m.clone()
        c.apply_to_device(th, v, fused=fused)
        assert float((v[:64] - m[:64]).abs().max()) > 1e-6
        inv.apply_to_device(th_inv, v, fused=fused)
        v.sub_(m)
        torch.cuda.synchronize()
        assert float(v.abs().max()) < 1e-11
        del v
    del m
    torch.cuda.empty_cache()
