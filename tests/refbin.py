"""Bincode 1.3 writer for the reference's index structs (test fixtures).

The reference dumps BruteForceIndex / PQIndex / IVFPQIndex<f32, usize> with
bincode's default encoding (src/index/bruteforce_idx.rs:84-106,
pq_idx.rs:243-265, 488-523): little-endian, usize as u64, Vec<T> as a u64
length and the elements, Option<T> as a u8 tag and the value, bool as u8,
Box<T> as T, a unit Metric variant as its u32 index, struct fields in
declaration order.  The reference cannot be built here, so files in that
layout are written from oracle-built indexes to exercise the library's
loader (hora_load_reference).
"""
import struct

import numpy as np


class W:
    def __init__(self):
        self.parts = []

    def u64(self, v):
        self.parts.append(struct.pack("<Q", int(v)))

    def u32(self, v):
        self.parts.append(struct.pack("<I", int(v)))

    def u8(self, v):
        self.parts.append(struct.pack("<B", int(v)))

    def f32s(self, a):
        a = np.ascontiguousarray(a, np.float32)
        self.u64(a.size)
        self.parts.append(a.tobytes())

    def u64s(self, a):
        a = np.ascontiguousarray(a, np.uint64)
        self.u64(a.size)
        self.parts.append(a.astype("<u8").tobytes())

    def nodes(self, rows, ids):
        # Vec<Node<f32, usize>>: { vectors: Vec<f32>, idx: Option<usize> }
        self.u64(len(rows))
        for r, i in zip(rows, ids):
            self.f32s(r)
            if i is None:
                self.u8(0)
            else:
                self.u8(1)
                self.u64(i)

    def bytes(self):
        return b"".join(self.parts)


def brute_force(rows, ids, metric):
    """BruteForceIndex { nodes (skipped), tmp_nodes, mt, dimension }."""
    w = W()
    w.nodes(rows, ids)
    w.u32(metric)
    w.u64(rows.shape[1])
    return w.bytes()


def _ranges(dim, n_sub):
    sd = dim // n_sub
    r = dim % sd
    out = []
    for i in range(n_sub):
        if i < r:
            b, e = i * (sd + 1), (i + 1) * (sd + 1)
        else:
            b, e = r * (sd + 1) + (i - r) * sd, r * (sd + 1) + (i + 1 - r) * sd
        out.append((b, e))
    return out


def _pq_struct(w, dim, n_sub, sub_bits, train_epoch, books, rows, ids, codes, residual, metric):
    """PQIndex fields in declaration order (pq_idx.rs:21-43).  books is
    [n_sub][K][dmax] (trimmed to each subspace's length), codes [n][n_sub]."""
    K = 1 << sub_bits
    rg = _ranges(dim, n_sub)
    w.u64(dim)
    w.u64(n_sub)
    w.u64(dim // n_sub)
    w.u64(len(rg))  # _dimension_range: Vec<Vec<usize>>
    for b, e in rg:
        w.u64s([b, e])
    w.u64(sub_bits)
    w.u64((sub_bits + 7) // 8)
    w.u64(K)
    w.u64(((sub_bits + 7) // 8) * n_sub)
    w.u64(train_epoch)
    trained = books is not None
    if trained:
        w.u64(n_sub)  # _centers: Vec<Vec<Vec<f32>>>
        for m, (b, e) in enumerate(rg):
            w.u64(K)
            for j in range(K):
                w.f32s(books[m][j][: e - b])
    else:
        w.u64(0)
    w.u8(1 if trained else 0)
    w.u8(1 if residual is not None else 0)
    w.f32s(residual if residual is not None else np.zeros(0, np.float32))
    w.u64(len(rows))
    w.u64(100000)
    w.nodes(rows, ids)  # _nodes
    if trained:
        w.u64(n_sub)  # _assigned_center: [n_sub][n]
        for m in range(n_sub):
            w.u64s(codes[:, m])
    else:
        w.u64(0)
    w.u32(metric)
    w.nodes(rows, ids)  # _nodes_tmp (the dump's copy)


def pq_index(rows, ids, n_sub, sub_bits, train_epoch, books, codes, metric):
    w = W()
    _pq_struct(w, rows.shape[1], n_sub, sub_bits, train_epoch, books, rows, ids, codes, None, metric)
    return w.bytes()


def ivfpq_index(rows, ids, n_sub, sub_bits, n_list, nprobe, train_epoch, ref, metric):
    """IVFPQIndex fields in declaration order (pq_idx.rs:266-289) from an
    oracle-built index `ref` (oracle.ivfpq_build)."""
    dim = rows.shape[1]
    w = W()
    for v in (dim, n_sub, dim // n_sub, sub_bits, (sub_bits + 7) // 8, 1 << sub_bits,
              ((sub_bits + 7) // 8) * n_sub, train_epoch, nprobe, n_list):
        w.u64(v)
    w.u64(n_list)  # _centers
    for c in range(n_list):
        w.f32s(ref["centers"][c])
    offs, items = ref["offsets"], ref["items"]
    w.u64(n_list)  # _ivflist
    for c in range(n_list):
        w.u64s(items[offs[c]:offs[c + 1]])
    w.u64(n_list)  # _pq_list
    for c in range(n_list):
        members = items[offs[c]:offs[c + 1]]
        _pq_struct(w, dim, n_sub, sub_bits, train_epoch,
                   ref["codebooks"][c] if ref["trained"][c] else None,
                   rows[members], [ids[i] for i in members], ref["codes"][offs[c]:offs[c + 1]],
                   ref["centers"][c], 3)
    w.u8(1)  # _is_trained
    w.u64(len(rows))
    w.u64(100000)
    w.nodes(rows, ids)  # _nodes
    w.u64(0)  # _assigned_center
    w.u32(metric)
    w.nodes(rows, ids)  # _nodes_tmp
    return w.bytes()
