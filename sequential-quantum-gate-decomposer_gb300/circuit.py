"""Gate structures: a drop-in for ``squander.Circuit`` (squander/gates/qgd_Circuit.py)
restricted to the hot-path gate set U3, RX, RY, RZ, CNOT, CZ, CRY and nested circuits.

Conventions follow SQUANDER: gates are appended in order and gates[0] acts first
(Gates_block::add_gate, src-cpp/gates/Gates_block.cpp:2500-2525); two-qubit gates take
``(target, control)``; parameters are contiguous in gate order, U3 stores
(theta/2, phi, lambda), the rotations store theta/2.  Every numerical method runs on the
GPU through libsqg.so.
"""
import ctypes

import numpy as np

from . import _device as dev
from . import _native

CZ, CNOT, U3, RY, RX, RZ, CRY = 4, 5, 7, 8, 9, 10, 14
GATE_NAMES = {CZ: "CZ", CNOT: "CNOT", U3: "U3", RY: "RY", RX: "RX", RZ: "RZ", CRY: "CRY"}
PARAM_NUM = {CZ: 0, CNOT: 0, U3: 3, RY: 1, RX: 1, RZ: 1, CRY: 1}


class NativeCircuit:
    """Owning wrapper of an ``sqg_circuit*`` handle."""

    def __init__(self, qbit_num, records):
        lib = _native.lib()
        recs = np.ascontiguousarray(np.asarray(records, dtype=np.int32).reshape(-1, 4))
        h = ctypes.c_void_p()
        _native.check(lib.sqg_circuit_create(int(qbit_num), recs.ctypes.data if recs.size else None, recs.shape[0],
                                             ctypes.byref(h)), "sqg_circuit_create")
        self.handle = h.value
        self.qbit_num = int(qbit_num)
        self.param_num = lib.sqg_circuit_param_num(self.handle)
        self.gate_num = recs.shape[0]
        self.records = recs

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                _native.lib().sqg_circuit_destroy(h)
            except Exception:
                pass
            self.handle = None


class Gate:
    """One gate of a Circuit (the gate objects of squander's gates_Wrapper): type, target,
    control (-1 when uncontrolled) and the start index of its parameters in the circuit that
    holds it.  Also reads as the gate dictionary of the decomposition classes' get_Gates
    ("type", "target_qbit", "control_qbit", "parameter_start_index")."""

    def __init__(self, gtype, target, control, param_start, index=-1):
        self.type, self.target, self.control = int(gtype), int(target), int(control)
        self.param_start = int(param_start)
        self._index = int(index)  # position among the top-level items of its circuit

    def get_Name(self):
        return GATE_NAMES[self.type]

    def get_Target_Qbit(self):
        return self.target

    def get_Control_Qbit(self):
        return self.control

    def get_Involved_Qbits(self):
        return sorted((self.target, self.control)) if self.control >= 0 else [self.target]

    def get_Parameter_Num(self):
        return PARAM_NUM[self.type]

    def get_Parameter_Start_Index(self):
        return self.param_start

    def _as_dict(self):
        d = {"type": GATE_NAMES[self.type], "target_qbit": self.target, "parameter_start_index": self.param_start}
        if self.control >= 0:
            d["control_qbit"] = self.control
        return d

    def __getitem__(self, key):
        return self._as_dict()[key]

    def __contains__(self, key):
        return key in self._as_dict()

    def get(self, key, default=None):
        return self._as_dict().get(key, default)

    def keys(self):
        return self._as_dict().keys()

    def __repr__(self):
        return "Gate(%s)" % self._as_dict()


class Circuit:
    """Ordered parametric gate list on ``qbit_num`` qubits (SQUANDER ``qgd_Circuit``), with
    nested sub-circuits (add_Circuit) kept as blocks of the top-level item list; the engine
    sees the flattened gate list."""

    def __init__(self, qbit_num):
        if int(qbit_num) < 1:
            raise ValueError("qbit_num must be positive")
        self.qbit_num = int(qbit_num)
        self._gates = []  # flattened (type, target, control)
        self._items = []  # top level: ("g", flat index) or ("c", sub-circuit, first flat index)
        self._native = None
        self._ws = dev.Workspace()
        self.min_fusion = -1
        self._pstart = 0  # parameter start index inside the circuit that holds this one
        self._index = -1

    # ---- structure -------------------------------------------------------------------
    def _check_qubit(self, q, what):
        if not (0 <= int(q) < self.qbit_num):
            raise ValueError("%s qubit index %d out of range for %d qubits" % (what, q, self.qbit_num))

    def _add(self, gtype, target, control=-1):
        self._check_qubit(target, "target")
        if control != -1:
            self._check_qubit(control, "control")
            if control == target:
                raise ValueError("control and target qubits must differ")
        self._items.append(("g", len(self._gates)))
        self._gates.append((gtype, int(target), int(control)))
        self._native = None

    def add_U3(self, target_qbit):
        self._add(U3, target_qbit)

    def add_RX(self, target_qbit):
        self._add(RX, target_qbit)

    def add_RY(self, target_qbit):
        self._add(RY, target_qbit)

    def add_RZ(self, target_qbit):
        self._add(RZ, target_qbit)

    def add_CNOT(self, target_qbit, control_qbit):
        self._add(CNOT, target_qbit, control_qbit)

    def add_CZ(self, target_qbit, control_qbit):
        self._add(CZ, target_qbit, control_qbit)

    def add_CRY(self, target_qbit, control_qbit):
        self._add(CRY, target_qbit, control_qbit)

    def add_adaptive(self, target_qbit, control_qbit):
        """The adaptive controlled rotation of the adaptive decomposer: a CRY, its activation
        function being the identity (src-cpp/common/common.cpp:35-38)."""
        self._add(CRY, target_qbit, control_qbit)

    def add_Circuit(self, other):
        """Append a sub-circuit as one block (Gates_block::add_gate of a nested block, its
        parameters contiguous after the ones before it)."""
        if other.qbit_num > self.qbit_num:
            raise ValueError("sub-circuit spans more qubits than the circuit")
        sub = other._copy()
        self._items.append(("c", sub, len(self._gates)))
        self._gates.extend(other._gates)
        self._native = None

    def add_Gate(self, gate):
        """Append a copy of a gate object taken from another circuit's get_Gates (a sub-circuit
        object is appended as a block)."""
        if isinstance(gate, Circuit):
            self.add_Circuit(gate)
        else:
            self._add(gate.type, gate.target, gate.control)

    def _copy(self):
        c = Circuit(self.qbit_num)
        c._gates = list(self._gates)
        c._items = [(it[0], it[1]._copy(), it[2]) if it[0] == "c" else it for it in self._items]
        c.min_fusion = self.min_fusion
        return c

    def _item_ranges(self):
        """(first flat gate, end flat gate) of every top-level item."""
        out = []
        for it in self._items:
            if it[0] == "g":
                out.append((it[1], it[1] + 1))
            else:
                out.append((it[2], it[2] + len(it[1]._gates)))
        return out

    def block_ends(self):
        """Flat gate index after every top-level item that is a block (sub-circuit); empty
        for a circuit without blocks."""
        if not any(it[0] == "c" for it in self._items):
            return []
        return [e for (_, e) in self._item_ranges()]

    def get_Qbit_Num(self):
        return self.qbit_num

    def get_Parameter_Num(self):
        return sum(PARAM_NUM[g[0]] for g in self._gates)

    def get_Gate_Num(self):
        return len(self._gates)

    def get_Gates(self):
        """Top-level gates (Gate objects) and sub-circuits, each with its parameter start index
        in this circuit (qgd_Circuit.get_Gates)."""
        out, p = [], 0
        for k, it in enumerate(self._items):
            if it[0] == "g":
                t, tg, c = self._gates[it[1]]
                out.append(Gate(t, tg, c, p, k))
                p += PARAM_NUM[t]
            else:
                sub = it[1]
                sub._pstart, sub._index = p, k
                out.append(sub)
                p += sub.get_Parameter_Num()
        return out

    def get_Flat_Gates(self):
        """Every gate of the flattened circuit (Gate objects, parameter start index in this
        circuit)."""
        out, p = [], 0
        for k, (t, tg, c) in enumerate(self._gates):
            out.append(Gate(t, tg, c, p, k))
            p += PARAM_NUM[t]
        return out

    def get_Involved_Qbits(self):
        return self.get_Qbits()

    def Remap_Qbits(self, qbit_map, qbit_num=None):
        """New circuit with qubit q of every gate moved to qbit_map[q] (a dict {initial:
        remapped} as in qgd_Circuit.Remap_Qbits, or a sequence), on qbit_num qubits
        (default: this circuit's)."""
        n = self.qbit_num if qbit_num is None else int(qbit_num)
        m = dict(qbit_map) if isinstance(qbit_map, dict) else {q: int(v) for q, v in enumerate(qbit_map)}
        out = Circuit(n)
        for it in self._items:
            if it[0] == "c":
                out.add_Circuit(it[1].Remap_Qbits(m, n))
                continue
            t, tg, c = self._gates[it[1]]
            if tg not in m or (c >= 0 and c not in m):
                raise ValueError("qbit_map does not cover every qubit of the circuit")
            out._add(t, int(m[tg]), int(m[c]) if c >= 0 else -1)
        return out

    def get_Qbits(self):
        """Sorted qubit indices the gates act on."""
        return sorted({q for _, tg, c in self._gates for q in ((tg, c) if c >= 0 else (tg,))})

    def _gate_qubits(self, k):
        """Qubits of top-level item k (a sub-circuit: all qubits of its gates)."""
        it = self._items[k]
        if it[0] == "c":
            return tuple(it[1].get_Qbits())
        _, tg, c = self._gates[it[1]]
        return (tg, c) if c >= 0 else (tg,)

    def _item_index(self, gate):
        k = gate if isinstance(gate, (int, np.integer)) else getattr(gate, "_index", -1)
        if not 0 <= k < len(self._items):
            raise ValueError("the gate is not a top-level item of this circuit")
        return int(k)

    def get_Parents(self, gate):
        """Indices of the top-level items that last act, before `gate` (an index or an object
        from get_Gates), on each of its qubits (Gates_block::determine_parents)."""
        gate = self._item_index(gate)
        out = set()
        for q in self._gate_qubits(gate):
            for k in range(gate - 1, -1, -1):
                if q in self._gate_qubits(k):
                    out.add(k)
                    break
        return sorted(out)

    def get_Children(self, gate):
        """Indices of the top-level items that next act, after `gate`, on each of its qubits
        (Gates_block::determine_children)."""
        gate = self._item_index(gate)
        out = set()
        for q in self._gate_qubits(gate):
            for k in range(gate + 1, len(self._items)):
                if q in self._gate_qubits(k):
                    out.add(k)
                    break
        return sorted(out)

    def get_Gate_Nums(self):
        nums = {}
        for t, _, _ in self._gates:
            nums[GATE_NAMES[t]] = nums.get(GATE_NAMES[t], 0) + 1
        return nums

    def get_Parameter_Start_Index(self):
        return self._pstart

    def set_min_fusion(self, min_fusion):
        """Recorded for API compatibility: the engine always applies the whole circuit to
        shared-memory column tiles, which subsumes SQUANDER's k-qubit fusion."""
        self.min_fusion = int(min_fusion)

    def gate_records(self):
        """(L, 4) int32 array of (type, target, control, param_start)."""
        recs, p = [], 0
        for t, tg, c in self._gates:
            recs.append((t, tg, c, p))
            p += PARAM_NUM[t]
        return np.asarray(recs, dtype=np.int32).reshape(-1, 4)

    def native(self):
        """The engine's handle of the flattened circuit; a circuit of blocks (a partitioned
        circuit) also hands its block boundaries to the fused state-vector plan."""
        if self._native is None:
            nc = NativeCircuit(self.qbit_num, self.gate_records())
            ends = self.block_ends()
            if ends:
                arr = np.ascontiguousarray(ends, dtype=np.int32)
                _native.check(_native.lib().sqg_circuit_set_partitions(nc.handle, arr.ctypes.data, arr.size),
                              "sqg_circuit_set_partitions")
            self._native = nc
        return self._native

    # ---- device-level operations (torch CUDA tensors in, results in place) -----------
    def _params_dev(self, parameters):
        p = dev.to_device_real(parameters).reshape(-1)
        if p.numel() != self.get_Parameter_Num():
            raise ValueError("expected %d parameters, got %d" % (self.get_Parameter_Num(), p.numel()))
        return p

    def apply_to_device(self, params_dev, mtx_dev, fused=True, stream=None):
        """In place M <- C(params) M for a CUDA complex128 tensor (rows x cols, or a batch
        (B, rows, cols) with params (B, P))."""
        nc = self.native()
        B = mtx_dev.shape[0] if mtx_dev.dim() == 3 else 1
        rows, cols = mtx_dev.shape[-2], mtx_dev.shape[-1]
        if rows != (1 << self.qbit_num):
            raise ValueError("Gates_block::apply_to: Wrong input size in Gates_block gate apply.")
        if not mtx_dev.is_contiguous():
            raise ValueError("matrix must be contiguous")
        ws_bytes = _native.lib().sqg_apply_workspace_bytes(nc.handle, B)
        ws = self._ws.get(ws_bytes)
        dev.after_current(stream)
        _native.check(_native.lib().sqg_apply(nc.handle, dev.ptr(params_dev) if params_dev.numel() else None, B,
                                              dev.ptr(mtx_dev), cols, cols, rows * cols, 1 if fused else 0,
                                              dev.ptr(ws), ws.numel(), dev.stream_ptr(stream)), "sqg_apply")
        return mtx_dev

    def apply_state_device(self, params_dev, states_dev, fused=True, stream=None):
        """In place psi <- C(params) psi for CUDA complex128 state vectors (2^n,) or a batch
        (B, 2^n) with params (B, P); up to 30 qubits (sqg_apply_state)."""
        nc = self.native()
        B = states_dev.shape[0] if states_dev.dim() == 2 else 1
        if states_dev.shape[-1] != (1 << self.qbit_num):
            raise ValueError("Gates_block::apply_to: Wrong input size in Gates_block gate apply.")
        if not states_dev.is_contiguous():
            raise ValueError("state must be contiguous")
        lib = _native.lib()
        ws = self._ws.get(lib.sqg_state_workspace_bytes(nc.handle, B))
        dev.after_current(stream)
        _native.check(lib.sqg_apply_state(nc.handle, dev.ptr(params_dev) if params_dev.numel() else None, B,
                                          dev.ptr(states_dev), states_dev.shape[-1], 1 if fused else 0, dev.ptr(ws),
                                          ws.numel(), dev.stream_ptr(stream)), "sqg_apply_state")
        return states_dev

    def get_Second_Renyi_Entropy(self, parameters=None, input_state=None, qubit_list=None):
        """Second Renyi entropy -log Tr(rho^2) of the reduced density matrix of qubit_list (all
        qubits when None) of the circuit's output state for input_state (|0...0> when None)
        (qgd_Circuit.get_Second_Renyi_Entropy, Gates_block::get_second_Renyi_entropy,
        src-cpp/gates/Gates_block.cpp:3625-3650).  The state is transformed on the GPU; the
        purity is one matrix product of the state reshaped as (kept qubits) x (traced qubits)."""
        n = self.qbit_num
        if isinstance(qubit_list, (list, tuple)):
            if not all(isinstance(q, (int, np.integer)) for q in qubit_list):
                print("Elements of qbit_list should be integers")
                return None
            keep = sorted(set(int(q) for q in qubit_list))
        elif qubit_list is None:
            keep = list(range(n))
        else:
            print("Elements of qbit_list should be integers")
            return None
        if parameters is None:
            print("get_Second_Renyi_entropy: array of input parameters is None")
            return None
        if any(not 0 <= q < n for q in keep):
            raise ValueError("qubit index out of range")
        if input_state is None:
            psi = np.zeros(1 << n, dtype=np.complex128)
            psi[0] = 1.0
        else:
            psi = np.ascontiguousarray(np.asarray(input_state, dtype=np.complex128).reshape(-1))
            if psi.size != (1 << n):
                raise ValueError("input state must have 2**qbit_num amplitudes")
        torch = dev.torch
        v = dev.to_device_complex(psi)
        self.apply_state_device(self._params_dev(parameters), v)
        traced = [q for q in range(n) if q not in keep]
        axes = [n - 1 - q for q in keep] + [n - 1 - q for q in traced]  # amplitude index bit q = axis n-1-q
        M = v.reshape([2] * n).permute(axes).reshape(1 << len(keep), 1 << len(traced))
        rho = M @ M.conj().transpose(0, 1) if len(keep) <= len(traced) else M.conj().transpose(0, 1) @ M
        purity = float((rho.real * rho.real + rho.imag * rho.imag).sum().item())
        return -float(np.log(purity))

    def state_block_count(self):
        """Fused passes over a state vector (blocks of the state-vector plan)."""
        return _native.lib().sqg_state_block_count(self.native().handle)

    # ---- SQUANDER-compatible host API (numpy in, numpy out / in place) ---------------
    def get_Matrix(self, parameters_mtx, is_f32=False):
        if is_f32:
            raise NotImplementedError("the GB300 engine computes in FP64 only")
        self.native()
        params = self._params_dev(parameters_mtx)
        m = dev.torch.eye(1 << self.qbit_num, dtype=dev.torch.complex128, device="cuda")
        self.apply_to_device(params, m)
        return m.cpu().numpy()

    def _check_mtx(self, unitary_mtx):
        if not isinstance(unitary_mtx, np.ndarray) or unitary_mtx.dtype != np.complex128:
            raise TypeError("input matrix must be a complex128 numpy array")
        if unitary_mtx.ndim == 1:
            unitary_mtx = unitary_mtx.reshape(-1, 1)
        if unitary_mtx.shape[0] != (1 << self.qbit_num):
            raise ValueError("Gates_block::apply_to: Wrong input size in Gates_block gate apply.")
        return unitary_mtx

    def apply_to(self, parameters_mtx, unitary_mtx, parallel=1, is_f32=False):
        """In place ``unitary_mtx <- C(parameters) unitary_mtx`` (qgd_Circuit.py:546)."""
        if is_f32:
            raise NotImplementedError("the GB300 engine computes in FP64 only")
        view = self._check_mtx(unitary_mtx)
        if np.asarray(parameters_mtx).dtype != np.float64:
            raise TypeError("parameters must be float64")
        params = self._params_dev(parameters_mtx)
        if view.shape[1] == 1:
            # state vector (the reference's state-vector kernels): any register up to 30 qubits
            psi = dev.to_device_complex(np.ascontiguousarray(view.reshape(-1)))
            self.apply_state_device(params, psi)
            view[...] = psi.cpu().numpy().reshape(-1, 1)
            return
        m = dev.to_device_complex(np.ascontiguousarray(view))
        self.apply_to_device(params, m)
        view[...] = m.cpu().numpy()

    def apply_to_list(self, inputs, parameters_mtx, parallel=1, is_f32=False):
        """Applies the circuit in place to every matrix of `inputs` (qgd_Circuit.py:572);
        inputs of one shape go through a single batched launch."""
        if is_f32:
            raise NotImplementedError("the GB300 engine computes in FP64 only")
        params = self._params_dev(parameters_mtx)
        groups = {}
        for i, m in enumerate(inputs):
            v = self._check_mtx(m)
            groups.setdefault(v.shape, []).append(i)
        for shape, idx in groups.items():
            stack = dev.torch.from_numpy(np.stack([np.ascontiguousarray(self._check_mtx(inputs[i])) for i in idx]))
            d = stack.cuda()
            self.apply_to_device(params.reshape(1, -1).expand(len(idx), -1).contiguous(), d)
            host = d.cpu().numpy()
            for k, i in enumerate(idx):
                self._check_mtx(inputs[i])[...] = host[k]

    def apply_from_right(self, parameters_mtx, unitary_mtx, parallel=1, is_f32=False):
        """In place ``unitary_mtx <- unitary_mtx C(parameters)`` (qgd_Circuit.py:559)."""
        if is_f32:
            raise NotImplementedError("the GB300 engine computes in FP64 only")
        if not isinstance(unitary_mtx, np.ndarray) or unitary_mtx.dtype != np.complex128:
            raise TypeError("input matrix must be a complex128 numpy array")
        if unitary_mtx.shape[-1] != (1 << self.qbit_num):
            raise ValueError("Gates_block::apply_from_right: Wrong matrix size")
        params = self._params_dev(parameters_mtx)
        nc = self.native()
        m = dev.to_device_complex(np.ascontiguousarray(unitary_mtx))
        ws = self._ws.get(_native.lib().sqg_apply_workspace_bytes(nc.handle, 1))
        _native.check(_native.lib().sqg_apply_from_right(nc.handle, dev.ptr(params) if params.numel() else None,
                                                         dev.ptr(m), m.shape[0], m.shape[1], dev.ptr(ws),
                                                         ws.numel(), dev.stream_ptr()), "sqg_apply_from_right")
        unitary_mtx[...] = m.cpu().numpy()

    def apply_to_combined(self, parameters_mtx, unitary_mtx, parallel=1, is_f32=False):
        """[C U, dC/dp_0 U, ...] (qgd_Circuit.py:597)."""
        if is_f32:
            raise NotImplementedError("the GB300 engine computes in FP64 only")
        if np.asarray(parameters_mtx).dtype != np.float64:
            raise TypeError("parameters must be float64")
        view = self._check_mtx(unitary_mtx)
        params = self._params_dev(parameters_mtx)
        out = combined_unitary_device(self.native(), params, dev.to_device_complex(np.ascontiguousarray(view)),
                                      self._ws)
        host = out.cpu().numpy()
        return [host[k] for k in range(host.shape[0])]

    def apply_derivate_to(self, parameters_mtx, unitary_mtx, parallel=1, is_f32=False):
        """[dC/dp_k U for every parameter] (qgd_Circuit.py:583)."""
        return self.apply_to_combined(parameters_mtx, unitary_mtx, parallel, is_f32)[1:]


def combined_unitary_device(nc, params_dev, target_dev, ws):
    """(P+1, rows, cols) CUDA tensor: the forward matrix and every derivative matrix."""
    rows, cols = target_dev.shape
    out = dev.torch.empty((nc.param_num + 1, rows, cols), dtype=dev.torch.complex128, device="cuda")
    buf = ws.get(_native.lib().sqg_apply_workspace_bytes(nc.handle, 1))
    _native.check(_native.lib().sqg_combined_unitary(nc.handle, dev.ptr(params_dev) if params_dev.numel() else None,
                                                     dev.ptr(target_dev), cols, dev.ptr(out), dev.ptr(buf),
                                                     buf.numel(), dev.stream_ptr()), "sqg_combined_unitary")
    return out
