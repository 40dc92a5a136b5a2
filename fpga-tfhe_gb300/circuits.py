"""Circuit builders for the gate server (gate lists of tfhe_gpu_server_submit)
and a plaintext evaluator to check results.

Gate tuple: (type, in0, in1, in2).  Types 0..9 are the two-input gates of
tfhe_gpu_gate (NAND, AND, OR, XOR, XNOR, NOR, ANDNY, ANDYN, ORNY, ORYN),
10 = MUX (in0 ? in1 : in2), 11 = NOT, 12 = COPY, 13 = CONSTANT (in0 = bit).
Wire ids: inputs first, then one wire per gate in list order.
"""
import numpy as np

NAND, AND, OR, XOR, XNOR, NOR, ANDNY, ANDYN, ORNY, ORYN, MUX, NOT, COPY, CONST = range(14)


class Builder:
    def __init__(self, ninputs):
        self.ninputs = ninputs
        self.gates = []

    def gate(self, t, a=-1, b=-1, c=-1):
        self.gates.append((t, a, b, c))
        return self.ninputs + len(self.gates) - 1

    def array(self):
        return np.array(self.gates, np.int32).reshape(-1, 4)


def ripple_carry_adder(bits):
    """a + b over `bits` bits: inputs a[0..bits), b[0..bits) (LSB first);
    outputs sum[0..bits) and the carry.  5 gates per bit (XOR, XOR, AND, AND,
    OR); depth 2 per bit along the carry chain."""
    B = Builder(2 * bits)
    a = list(range(bits))
    b = list(range(bits, 2 * bits))
    outs = []
    carry = None
    for i in range(bits):
        t = B.gate(XOR, a[i], b[i])
        g = B.gate(AND, a[i], b[i])
        if carry is None:
            outs.append(t)
            carry = g
            continue
        s = B.gate(XOR, t, carry)
        p = B.gate(AND, t, carry)
        carry = B.gate(OR, g, p)
        outs.append(s)
    outs.append(carry)
    return B.array(), 2 * bits, outs


def comparator(bits):
    """1 if b > a else 0, over `bits` bits (LSB first), the compare_bit chain
    of test_bench/server/cloud.c:9-31: carry = MUX(XNOR(a_i, b_i), carry, b_i)
    from the LSB up, starting from the constant 0."""
    B = Builder(2 * bits)
    carry = B.gate(CONST, 0)
    for i in range(bits):
        eq = B.gate(XNOR, i, bits + i)
        carry = B.gate(MUX, eq, carry, bits + i)
    return B.array(), 2 * bits, [carry]


def multiplexer(bits):
    """sel ? x : y over `bits` bits: inputs sel, x[0..bits), y[0..bits)."""
    B = Builder(1 + 2 * bits)
    outs = [B.gate(MUX, 0, 1 + i, 1 + bits + i) for i in range(bits)]
    return B.array(), 1 + 2 * bits, outs


_FN = [lambda x, y: 1 - (x & y), lambda x, y: x & y, lambda x, y: x | y, lambda x, y: x ^ y,
       lambda x, y: 1 - (x ^ y), lambda x, y: 1 - (x | y), lambda x, y: (1 - x) & y,
       lambda x, y: x & (1 - y), lambda x, y: (1 - x) | y, lambda x, y: x | (1 - y)]


def evaluate(gates, inputs, outputs):
    """Plaintext evaluation of a gate list on input bits."""
    w = list(int(v) for v in inputs)
    for t, a, b, c in np.asarray(gates).reshape(-1, 4):
        if t <= 9:
            w.append(_FN[t](w[a], w[b]))
        elif t == MUX:
            w.append(w[b] if w[a] else w[c])
        elif t == NOT:
            w.append(1 - w[a])
        elif t == COPY:
            w.append(w[a])
        else:
            w.append(int(a))
    return np.array([w[o] for o in outputs], np.int32)


def bootstraps(gates):
    """Bootstraps a gate list costs (MUX = 2, NOT/COPY/CONSTANT = 0)."""
    t = np.asarray(gates).reshape(-1, 4)[:, 0]
    return int((t <= 9).sum() + 2 * (t == MUX).sum())
