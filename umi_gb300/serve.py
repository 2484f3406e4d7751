"""Multi-stream serving of a batched image operator.

A request is one batch: an input image (and an auxiliary one: weights or the
right feature map) per slot, every slot of fixed shape, through one batched
operator (bilateral, per-pixel wfilter3x3, cost volume).  ``BatchServer``
keeps ``instances`` copies of the device buffers, each with the operator
recorded into its own batch graph (``umi_batch_graph_*``) and its own CUDA
stream.  ``submit`` puts a request on the next instance in turn: the host
arrays are copied into that instance's pinned staging buffers, uploaded,
the graph is replayed and the outputs are downloaded, all queued on the
instance's stream, so up to ``instances`` requests are in flight and the
transfers of one overlap the compute of another.  ``result`` waits for a
request and returns its outputs (copies).
"""
from __future__ import annotations

import numpy as np

import umi_gb300 as U


class BatchServer:
    """slots: list of (in_shape, aux_shape or None, out_shape) float32
    images; op / params / variant as ``umi_gb300.batch_run``."""

    def __init__(self, op: int, slots, params=None, variant: int = -1, instances: int = 2, device="cuda"):
        import torch
        if instances < 1:
            raise ValueError("at least one instance")
        if not slots:
            raise ValueError("no slots")
        self.op, self.slots, self.params, self.variant = op, list(slots), params, variant
        self.device = torch.device(device)
        self.inst = []
        for _ in range(instances):
            d = {"stream": torch.cuda.Stream(device=self.device), "event": None, "ticket": None}
            d["d_in"] = [torch.empty(s[0], dtype=torch.float32, device=self.device) for s in self.slots]
            d["d_aux"] = [torch.empty(s[1], dtype=torch.float32, device=self.device) if s[1] else None
                          for s in self.slots]
            d["d_out"] = [torch.empty(s[2], dtype=torch.float32, device=self.device) for s in self.slots]
            d["h_in"] = [torch.empty(s[0], dtype=torch.float32).pin_memory() for s in self.slots]
            d["h_aux"] = [torch.empty(s[1], dtype=torch.float32).pin_memory() if s[1] else None for s in self.slots]
            d["h_out"] = [torch.empty(s[2], dtype=torch.float32).pin_memory() for s in self.slots]
            g = U.BatchGraph()
            g.add(op, list(zip(d["d_in"], d["d_aux"], d["d_out"])), params, variant)
            d["graph"] = g
            self.inst.append(d)
        self.next = 0
        self.tickets = 0
        self.done = {}  # finished results not yet collected: ticket -> outputs

    def _collect(self, d):
        if d["ticket"] is not None:
            d["event"].synchronize()
            self.done[d["ticket"]] = [t.numpy().copy() for t in d["h_out"]]
            d["ticket"] = None

    def submit(self, inputs, auxes=None) -> int:
        """Queue one request (one array per slot, and one auxiliary array per
        slot that has one); returns its ticket."""
        import torch
        if len(inputs) != len(self.slots) or (auxes is not None and len(auxes) != len(self.slots)):
            raise ValueError(f"expected {len(self.slots)} images per request")
        d = self.inst[self.next]
        self.next = (self.next + 1) % len(self.inst)
        self._collect(d)  # the instance's previous request is done and its outputs are kept
        for k, s in enumerate(self.slots):
            np.copyto(d["h_in"][k].numpy(), np.asarray(inputs[k], dtype=np.float32).reshape(s[0]))
            if s[1]:
                if auxes is None or auxes[k] is None:
                    raise ValueError(f"slot {k} needs an auxiliary image")
                np.copyto(d["h_aux"][k].numpy(), np.asarray(auxes[k], dtype=np.float32).reshape(s[1]))
        st = d["stream"]
        with torch.cuda.stream(st):
            for k in range(len(self.slots)):
                d["d_in"][k].copy_(d["h_in"][k], non_blocking=True)
                if d["d_aux"][k] is not None:
                    d["d_aux"][k].copy_(d["h_aux"][k], non_blocking=True)
            d["graph"].launch(st)
            for k in range(len(self.slots)):
                d["h_out"][k].copy_(d["d_out"][k], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(st)
        d["event"] = ev
        self.tickets += 1
        d["ticket"] = self.tickets
        return self.tickets

    def result(self, ticket: int, copy: bool = True):
        """The outputs (one array per slot) of a submitted request.  copy=False
        returns views of the instance's pinned output buffers instead: no host
        copy, valid until the instance takes another request (``instances``
        submissions later)."""
        if ticket in self.done:
            return self.done.pop(ticket)
        for d in self.inst:
            if d["ticket"] == ticket:
                if copy:
                    self._collect(d)
                    return self.done.pop(ticket)
                d["event"].synchronize()
                d["ticket"] = None
                return [t.numpy() for t in d["h_out"]]
        raise KeyError(f"unknown or already collected ticket {ticket}")

    def drain(self):
        """Waits for every request in flight."""
        for d in self.inst:
            self._collect(d)

    def close(self):
        self.drain()
        for d in self.inst:
            d["graph"].close()
