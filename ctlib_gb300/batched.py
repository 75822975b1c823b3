"""Ragged batches: slices with different geometries processed together.

    rb = RaggedBatch([options_0, options_1, ...])      # one options vector per slice (fp32; dtype=torch.float64 too)
    sinos = rb.projection([img_0, img_1, ...])          # list of 1 x 1 x V_i x D_i
    recs = rb.fbp(sinos)                                 # list of 1 x 1 x H_i x W_i

Every stage of an operator is a single launch over all slices
(``ctgb_ragged_run``): the task list is built once, longest tasks first, and
per-slice pointers and plans are kernel parameters, so a run can be captured in
a CUDA graph: ``rb.graphed(op, inputs)`` returns a replayable callable over
static input/output buffers.

``rb.graphed(op, inputs, branches=k)`` with k > 0 instead captures each
slice's own per-slice launches (the staged image gather included) on k
parallel branches of the graph, slices assigned longest first to the least
loaded branch: no launch or plan overhead per call, and small slices overlap
one another. ``branches=0`` captures the one-launch-per-stage form, and the
default ``branches="auto"`` the form the autotuner measured fastest for this
batch (``tune.tune_ragged``, cached per batch signature).
"""

from __future__ import annotations

import ctypes

import torch

from . import _native as N
from . import tune
from .ops import _FN, get_plan

_OPS = {"projection": N.OP_PROJECTION, "projection_t": N.OP_PROJECTION_T, "backprojection": N.OP_BACKPROJECTION,
        "backprojection_t": N.OP_BACKPROJECTION_T, "fbp": N.OP_FBP}


class RaggedBatch:
    def __init__(self, options_list, device=None, dtype=torch.float32):
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        if dtype not in (torch.float32, torch.float64):
            raise ValueError(f"dtype must be float32 or float64, got {dtype}")
        self.device = torch.device(device)
        self.dtype = dtype
        idx = self.device.index if self.device.index is not None else torch.cuda.current_device()
        self.plans = [get_plan(o, dtype, self.device) for o in options_list]
        n = len(self.plans)
        arr = (ctypes.c_void_p * n)(*[p.handle.value for p in self.plans])
        h = ctypes.c_void_p()
        rc = N.lib().ctgb_ragged_create(ctypes.byref(h), arr, n, idx)
        N.check(rc, "ragged batch")
        self.handle = h
        self.n = n

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            try:
                N._lib.ctgb_ragged_destroy(h)
            except Exception:
                pass
            self.handle = None

    def _shapes(self, op):
        if op in (N.OP_PROJECTION, N.OP_BACKPROJECTION_T):
            return [(1, 1, p.views, p.dets) for p in self.plans], [(1, 1, p.height, p.width) for p in self.plans]
        return [(1, 1, p.height, p.width) for p in self.plans], [(1, 1, p.views, p.dets) for p in self.plans]

    def workspace_bytes(self, op: int) -> int:
        return int(N.lib().ctgb_ragged_workspace_size(self.handle, op))

    def run(self, op, inputs, outputs=None, workspace=None, stream=None):
        op = _OPS.get(op, op)
        if len(inputs) != self.n:
            raise ValueError(f"expected {self.n} slices, got {len(inputs)}")
        out_shapes, in_shapes = self._shapes(op)
        for i, (x, shp) in enumerate(zip(inputs, in_shapes)):
            if not (x.is_cuda and x.is_contiguous() and x.dtype == self.dtype):
                raise RuntimeError(f"slice {i}: input must be a contiguous {self.dtype} CUDA tensor")
            if tuple(x.shape) != shp and x.numel() != shp[2] * shp[3]:
                raise ValueError(f"slice {i}: input shape {tuple(x.shape)}, expected {shp}")
        if outputs is None:
            outputs = [torch.empty(s, dtype=self.dtype, device=self.device) for s in out_shapes]
        nbytes = self.workspace_bytes(op)
        if workspace is None:
            workspace = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        ins = (ctypes.c_void_p * self.n)(*[x.data_ptr() for x in inputs])
        outs = (ctypes.c_void_p * self.n)(*[y.data_ptr() for y in outputs])
        rc = N.lib().ctgb_ragged_run(self.handle, op, ins, outs, workspace.data_ptr(), nbytes, stream.cuda_stream)
        N.check(rc, "ragged run")
        return outputs

    def projection(self, images):
        return self.run(N.OP_PROJECTION, images)

    def projection_t(self, sinos):
        return self.run(N.OP_PROJECTION_T, sinos)

    def backprojection(self, sinos):
        return self.run(N.OP_BACKPROJECTION, sinos)

    def backprojection_t(self, images):
        return self.run(N.OP_BACKPROJECTION_T, images)

    def fbp(self, sinos):
        return self.run(N.OP_FBP, sinos)

    def graphed(self, ops, inputs, branches="auto"):
        """Capture `ops` (one op name or a chain such as ("projection", "fbp"),
        each op consuming the previous one's outputs) into a CUDA graph over
        static copies of `inputs`. Returns (replay, static_inputs, outputs):
        copy new data into static_inputs, call replay(), read outputs.
        branches = k > 0: the slices' own launches on k parallel graph
        branches; branches = 0: one launch per stage over all slices;
        "auto" (default): the form the autotuner picked for this batch and
        chain (tune.tune_ragged), timing the forms first if none is cached."""
        if isinstance(ops, str):
            ops = (ops,)
        if branches == "auto":
            branches = tune.ragged_cached(self, ops)
            if branches is None:
                branches = tune.tune_ragged(self, ops, inputs)["branches"]
        if not isinstance(branches, int) or branches < 0:
            raise ValueError("branches must be 'auto' or an int >= 0")
        static_in = [x.clone() for x in inputs]
        if branches:
            return self._graphed_branches(ops, static_in, branches)
        bufs, cur = [], static_in
        for name in ops:
            op = _OPS[name]
            out_shapes, _ = self._shapes(op)
            outs = [torch.empty(s, dtype=self.dtype, device=self.device) for s in out_shapes]
            ws = torch.empty(max(self.workspace_bytes(op), 1), dtype=torch.uint8, device=self.device)
            bufs.append((op, cur, outs, ws))
            cur = outs
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for op, i, o, w in bufs:  # warm-up outside capture
                self.run(op, i, o, w, stream=side)
        torch.cuda.current_stream(self.device).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for op, i, o, w in bufs:
                self.run(op, i, o, w)
        # the captured kernels read this batch's device tables (task lists, plan
        # copies, offsets), which ctgb_ragged_destroy frees: the replay holds
        # the batch itself, not only the buffers
        return _replayer(graph, (self, bufs)), static_in, cur

    def _graphed_branches(self, ops, static_in, branches):
        chains, work = [], []
        for i, plan in enumerate(self.plans):
            cur, chain = static_in[i], []
            for name in ops:
                op = _OPS[name]
                tune.apply_cached(plan, op, 1)  # the schedule a per-slice call would use
                out_shapes, _ = self._shapes(op)
                out = torch.empty(out_shapes[i], dtype=self.dtype, device=self.device)
                nbytes = plan.workspace_bytes(op, 1)
                ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=self.device)
                chain.append((plan, op, cur, out, ws, nbytes))
                cur = out
            chains.append(chain)
            work.append(plan.views * plan.dets * max(plan.height, plan.width))
        lanes = assign_branches(work, branches)
        streams = [torch.cuda.Stream(self.device) for _ in range(branches)]

        def issue():
            main = torch.cuda.current_stream(self.device)
            for st, lane in zip(streams, lanes):
                st.wait_stream(main)
                for i in lane:
                    for plan, op, x, y, ws, nbytes in chains[i]:
                        rc = _FN[op](plan.handle, x.data_ptr(), y.data_ptr(), 1, ws.data_ptr(), nbytes,
                                     st.cuda_stream)
                        N.check(rc, "ragged branch")
            for st in streams:
                main.wait_stream(st)

        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            issue()  # warm-up outside capture
        torch.cuda.current_stream(self.device).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            issue()
        return _replayer(graph, (chains, streams)), static_in, [c[-1][3] for c in chains]


def _replayer(graph, buffers):
    """graph.replay, holding what the graph reads and writes: its intermediate
    outputs and workspaces, and the plans or ragged batch whose device tables
    its kernels read. The graph owns none of that memory; once freed, the
    caching allocator would hand the tensors to others and a destroyed plan or
    batch would leave the kernels reading released device memory."""

    def replay():
        graph.replay()

    replay.graph, replay.buffers = graph, buffers
    return replay


def assign_branches(work, branches: int):
    """Slices (by index) for each of `branches` graph branches: longest slice
    first, each to the branch with the least work so far (ties to the lower
    branch), so that the branches end close together."""
    if branches < 1:
        raise ValueError("branches must be >= 1")
    load, lanes = [0] * branches, [[] for _ in range(branches)]
    for i in sorted(range(len(work)), key=lambda j: -work[j]):
        b = min(range(branches), key=lambda k: load[k])
        load[b] += work[i]
        lanes[b].append(i)
    return lanes
