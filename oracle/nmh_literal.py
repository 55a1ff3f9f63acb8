"""Literal, step-by-step CPU emulation of cudaRebuildNMH (test infrastructure only).

kernels/rebuilder.cu cannot be compiled here (Thrust device code, <<<>>>
launches), so this module replays its kernel sequence on the host, one
function per kernel, with the same array state (indices, nodes, split list):
  sortTriangles        rebuilder.cu:262-289  two stable sorts + gathers
  swapMaxTriangleTPS   rebuilder.cu:127-151  (the deterministic variant; the
                       TPT variant, :93-125, computes the same on tie-free keys)
  updateNodesTPS       rebuilder.cu:171-187
  emitSplits           rebuilder.cu:189-215, 247-260 (+ thrust::copy_if)
  cudaRebuildNMH loop  rebuilder.cu:311-420
It pins the canonical build of aur_oracle.cpp: on inputs without key ties the
two must produce the same permutation. Small inputs only (Python loops).
"""
import numpy as np


def log2i(x):
    r = -1
    while x:
        x >>= 1
        r += 1
    return r


def exp2i(x):
    return 1 if x == 0 else 2 ** x


def calc_partition(N):
    n = N // 2
    H = log2i(n)
    s = exp2i(H - 1) - 1 if H >= 1 else 0
    S = exp2i(H) - 1
    O = max(0, (n - 1) - s - S)
    R = 2 * (s + O)
    L = 2 * (n - 1) - R
    return L, R


def triangle_bounds(V):
    V = np.asarray(V, np.float32).reshape(-1, 9)
    mn = [V[:, 3 * a:3 * a + 3].min(axis=1) for a in range(3)]
    mx = [V[:, 3 * a:3 * a + 3].max(axis=1) for a in range(3)]
    return mn, mx


def sort_triangles(keys, indices, nodes):
    count = indices.shape[0]
    permutation = np.arange(count)
    tempf = keys[indices]
    permutation = permutation[np.argsort(tempf, kind="stable")]
    tempi = nodes[permutation]
    permutation = permutation[np.argsort(tempi, kind="stable")]
    return indices[permutation].copy(), nodes[permutation].copy()


def swap_max_tps(keys, splits, indices, nodes):
    for index, size in splits:
        max_value = keys[indices[index + 1]]
        max_index = index + 1
        for i in range(index + 2, index + size):
            value = keys[indices[i]]
            if value > max_value:
                max_index, max_value = i, value
        if max_index != index + 1:
            indices[index + 1], indices[max_index] = indices[max_index], indices[index + 1]
            nodes[index + 1], nodes[max_index] = nodes[max_index], nodes[index + 1]


def update_nodes_tps(splits, done_nodes, nodes):
    for j, (index, size) in enumerate(splits):
        node_index = done_nodes + j
        nodes[index] = node_index
        nodes[index + 1] = node_index
        nodes[index + 2:index + size] = 2 * node_index + 1


def emit_splits(splits):
    pending = len(splits)
    out = {}
    generated = 0
    for j, (index, size) in enumerate(splits):
        if size <= 2:
            continue
        numL, numR = calc_partition(size)
        pL = index + 2 * (pending - j)
        pR = pL + numL
        out[2 * j] = (pL, numL)
        out[2 * j + 1] = (pR, numR)
        generated += (numL > 0) + (numR > 0)
    # thrust::copy_if over the first `generated` entries of outSplits
    return [out[i] for i in range(generated) if out[i][1] > 0]


def rebuild_nmh(V):
    """Returns indices: NMH position -> original triangle id."""
    V = np.asarray(V, np.float32).reshape(-1, 9)
    count = V.shape[0]
    assert count % 2 == 0 and count > 0
    num_levels = log2i(count // 2) + 1
    mn, mx = triangle_bounds(V)
    indices = np.arange(count, dtype=np.int64)
    nodes = np.zeros(count, dtype=np.int64)
    splits = [(0, count)]
    done_nodes = 0
    axis = 0
    for i in range(num_levels):
        indices, nodes = sort_triangles(mn[axis], indices, nodes)
        if i == num_levels - 1:
            break
        swap_max_tps(mx[axis], splits, indices, nodes)
        update_nodes_tps(splits, done_nodes, nodes)
        if i < max(0, num_levels - 2):
            new = emit_splits(splits)
            done_nodes += len(splits)
            splits = new
        axis = (axis + 1) % 3
    return indices.astype(np.uint32)


def has_key_ties(V):
    mn, mx = triangle_bounds(V)
    return any(np.unique(k).shape[0] != k.shape[0] for k in mn + mx)
