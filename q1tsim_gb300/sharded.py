"""A state of n qubits sharded over G = 2^g ranks, one GPU each.

The reference keeps one complex128 vector of 2^n amplitudes in host memory
(src/vectorstate.rs:24-53); one GB300 holds up to about 34 qubits in
complex64.  Above that the vector is split by its top g index bits: rank r
holds the amplitudes whose index is r * 2^L + i, i < 2^L, L = n - g, as an
engine state of L qubits.  Qubit q is index bit n-1-q (src/gates.rs:133-141),
so at the start qubits 0 .. g-1 are the "global" ones, selected by the rank.

Gates on local qubits run on each shard through the engine, with no
communication.  A gate on a global qubit first swaps that qubit with a
local one: ranks r and r ^ 2^j (j the global bit) exchange the half of
their shards in which the local bit differs from their own global bit
(torch.distributed send/recv: NCCL between GPUs, gloo between CPU
processes).  The highest free local position is taken, so for one column
the half is one contiguous block.  `pos[q]` records where logical qubit q
sits; the swap changes it, not the amplitudes' meaning.

Sampling (peek_all_into) first puts every qubit back at its own position,
so that shot k maps to the same outcome as in the unsharded state for the
same uniform: the shard weights are all-gathered, each rank takes the shots
whose uniform falls in its part of the prefix and samples its shard with
the uniforms rescaled into it, and the classical words are summed over the
ranks (each shot is filled by exactly one rank).

Only single-column states (before any measurement split) are sharded.
"""
import numpy as np

from .vectorstate import VectorState

SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


class _DeviceArray:
    """A raw device buffer seen by torch without a copy
    (__cuda_array_interface__)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


class EngineShard:
    """A rank's shard on its GPU: an engine state of L qubits whose
    amplitudes the exchange reads and writes in place
    (q1g_state_device_amplitudes / q1g_state_amplitudes_written)."""

    def __init__(self, nr_bits, nr_shots, precision):
        self.state = VectorState(nr_bits, nr_shots, precision)
        self.precision = precision

    def apply_gate(self, mat, bits):
        self.state.apply_gate(mat, bits)

    def amplitudes(self):
        import ctypes

        import torch

        from . import _lib
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        _lib.check(_lib.load().q1g_state_device_amplitudes(self.state._h, ctypes.byref(ptr), ctypes.byref(nbytes)),
                   "device_amplitudes")
        item = 16 if self.precision == "c128" else 8
        arr = _DeviceArray(ptr.value, nbytes.value // item, "<c16" if item == 16 else "<c8")
        return torch.as_tensor(arr, device="cuda")

    def amplitudes_written(self):
        import torch

        from . import _lib
        torch.cuda.current_stream().synchronize()
        _lib.check(_lib.load().q1g_state_amplitudes_written(self.state._h), "amplitudes_written")

    def column_norms(self):
        from . import _lib
        out = np.zeros(1, dtype=np.float64)
        _lib.check(_lib.load().q1g_state_column_norms(self.state._h, out.ctypes.data_as(_lib._dp), 1),
                   "column_norms")
        return out

    def peek_all_into(self, cbits, res, uniforms):
        self.state.peek_all_into(cbits, res, uniforms=uniforms)


class ShardedState:
    """State of nr_bits qubits over the ranks of `group` (a power of two),
    each rank's shard made by shard_factory(L, nr_shots, precision) (an
    EngineShard by default).  Starts in |0...0>."""

    def __init__(self, nr_bits, nr_shots=1, precision="c128", shard_factory=None, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        g = self.world.bit_length() - 1
        if self.world != 1 << g:
            raise ValueError("the number of ranks must be a power of two")
        if nr_bits - g < 2:
            raise ValueError("each shard needs at least 2 qubits")
        self.nr_bits, self.g, self.L = nr_bits, g, nr_bits - g
        self.nr_shots = nr_shots
        make = shard_factory or EngineShard
        self.shard = make(self.L, nr_shots, precision)
        self.pos = [nr_bits - 1 - q for q in range(nr_bits)]   # position of logical qubit q
        self.exchanges = 0                                       # half-shard exchanges so far
        if self.rank != 0:
            # |0...0> lives on rank 0; the other shards are zero
            a = self.shard.amplitudes()
            a.zero_()
            self.shard.amplitudes_written()

    # ------------------------------------------------------------ layout
    def _rank_bit(self, j):
        return (self.rank >> j) & 1

    def _qubit_at(self, p):
        return self.pos.index(p)

    def _swap_global_local(self, pg, pl):
        """Exchange physical positions pg (global) and pl (local): ranks
        r and r ^ 2^(pg-L) trade the half of their shard whose bit pl differs
        from their own bit pg-L."""
        import torch
        j = pg - self.L
        partner = self.rank ^ (1 << j)
        keep = self._rank_bit(j)
        a = self.shard.amplitudes()
        v = a.view(-1, 2, 1 << pl)[:, 1 - keep, :]      # the half that moves
        send = torch.view_as_real(v.contiguous())        # sent as (re, im) reals
        recv = torch.empty_like(send)
        ops = [self.dist.P2POp(self.dist.isend, send, partner, self.group),
               self.dist.P2POp(self.dist.irecv, recv, partner, self.group)]
        for req in self.dist.batch_isend_irecv(ops):
            req.wait()
        v.copy_(torch.view_as_complex(recv))
        self.shard.amplitudes_written()
        self.exchanges += 1
        qa, qb = self._qubit_at(pg), self._qubit_at(pl)
        self.pos[qa], self.pos[qb] = pl, pg

    def _swap_local(self, p1, p2):
        """Exchange local positions p1 and p2 with one swap pass on every
        shard."""
        self.shard.apply_gate(SWAP, [self.L - 1 - p1, self.L - 1 - p2])
        qa, qb = self._qubit_at(p1), self._qubit_at(p2)
        self.pos[qa], self.pos[qb] = p2, p1

    def _free_local(self, used):
        for p in range(self.L - 1, -1, -1):
            if p not in used:
                return p
        raise ValueError("gate acts on more qubits than a shard holds")

    def canonicalize(self):
        """Put every logical qubit q back at position n-1-q."""
        n, L = self.nr_bits, self.L
        for j in range(self.g):
            p = L + j
            want = n - 1 - p
            if self.pos[want] == p:
                continue
            if self.pos[want] >= L:      # at another global position: through a local one
                self._swap_global_local(self.pos[want], self._free_local(set()))
            self._swap_global_local(p, self.pos[want])
        for p in range(L):
            want = n - 1 - p
            if self.pos[want] != p:
                self._swap_local(p, self.pos[want])

    # ------------------------------------------------------------ QuState
    def apply_gate(self, mat, bits):
        """src/vectorstate.rs:166-178 on the sharded state."""
        mat = np.asarray(mat, dtype=np.complex128)
        bits = list(bits)
        if len(set(bits)) != len(bits) or any(b < 0 or b >= self.nr_bits for b in bits):
            raise ValueError(f"invalid qubits {bits}")
        used = {self.pos[b] for b in bits if self.pos[b] < self.L}
        for b in bits:
            if self.pos[b] >= self.L:
                pl = self._free_local(used)
                self._swap_global_local(self.pos[b], pl)
                used.add(pl)
        self.shard.apply_gate(mat, [self.L - 1 - self.pos[b] for b in bits])

    def peek_all_into(self, cbits, res, uniforms):
        """src/vectorstate.rs:395-400 on the sharded state, with the sorted
        uniforms given: the same words as the unsharded state."""
        import torch
        n, L = self.nr_bits, self.L
        if len(cbits) != n:
            raise ValueError("one classical bit per qubit")
        u = np.sort(np.asarray(uniforms, dtype=np.float64))
        if len(u) != self.nr_shots or len(res) < self.nr_shots:
            raise ValueError("one uniform and one result word per run")
        self.canonicalize()
        w = torch.tensor(self.shard.column_norms()[:1], dtype=torch.float64)
        ws = [torch.zeros(1, dtype=torch.float64) for _ in range(self.world)]
        dev = self.shard.amplitudes().device
        wd = w.to(dev)
        wsd = [x.to(dev) for x in ws]
        self.dist.all_gather(wsd, wd, group=self.group)
        weights = np.array([float(x.cpu()[0]) for x in wsd])
        total = weights.sum()
        lo = weights[:self.rank].sum()
        hi = lo + weights[self.rank]
        x = u * total
        mine = (x >= lo) & (x < hi) if self.rank < self.world - 1 else (x >= lo)
        words = np.zeros(len(u), dtype=np.int64)
        if mine.any() and weights[self.rank] > 0:
            # every shot gets a uniform inside this shard's range (clamped,
            # so the order stays sorted); only this rank's shots are kept
            ul = np.clip((x - lo) / weights[self.rank], 0.0, np.nextafter(1.0, 0.0))
            local_cbits = [cbits[n - 1 - p] for p in range(L - 1, -1, -1)]
            out = np.zeros(len(u), dtype=np.uint64)
            self.shard.peek_all_into(local_cbits, out, ul)
            gbits = 0
            for j in range(self.g):
                if self._rank_bit(j):
                    gbits |= 1 << cbits[n - 1 - (L + j)]
            words[mine] = (out[mine] | np.uint64(gbits)).astype(np.int64)
        t = torch.from_numpy(words).to(dev)
        self.dist.all_reduce(t, group=self.group)
        res[:len(u)] = t.cpu().numpy().astype(np.uint64)

    def states(self):
        """The full state in the qubits' own order, on every rank (for
        checks at small sizes: it gathers all shards)."""
        import torch
        self.canonicalize()
        a = torch.view_as_real(self.shard.amplitudes().contiguous())
        parts = [torch.empty_like(a) for _ in range(self.world)]
        self.dist.all_gather(parts, a, group=self.group)
        full = torch.view_as_complex(torch.cat(parts))
        return full.cpu().numpy().astype(np.complex128).reshape(-1, 1)
