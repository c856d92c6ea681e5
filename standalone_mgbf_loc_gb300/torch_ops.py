"""PyTorch operators over libmgbf's C-ABI: torch.ops.mgbf.*.

A thin extension layer for Python callers who work in torch terms: each
operator takes tensors and plain integers, and calls the same C entry point
as the MGBF / MGBFBatch classes (no second implementation, no CPU path).
Handles and batches are referred to by the integer id that register()
returns, because an operator's schema cannot carry Python objects.

    op = MGBF(cfg)
    hid = torch_ops.register(op)
    torch.ops.mgbf.filtering_procedure_(vall, hid, 6)     # in place, like filtering_procedure(6)

The operators mutate their field arguments in place (schema `Tensor(a!)`)
and have fake (meta) implementations, so tracing tools see the mutation and
the unchanged shapes.  They run on the current CUDA stream.
"""
from __future__ import annotations

import itertools
from typing import List, Union

import torch

from .mgbf import MGBF, MGBFBatch

_registry: dict = {}
_ids = itertools.count(1)


def register(obj: Union[MGBF, MGBFBatch]) -> int:
    """Make an MGBF handle or MGBFBatch reachable from torch.ops.mgbf.*;
    returns its id (valid until unregister)."""
    if not isinstance(obj, (MGBF, MGBFBatch)):
        raise TypeError("register() takes an MGBF or an MGBFBatch")
    i = next(_ids)
    _registry[i] = obj
    return i


def unregister(i: int) -> None:
    _registry.pop(int(i), None)


def _get(i: int, kind):
    obj = _registry.get(int(i))
    if not isinstance(obj, kind):
        raise ValueError(f"no registered {kind.__name__} with id {i}")
    return obj


@torch.library.custom_op("mgbf::filtering_procedure_", mutates_args=("vall",))
def filtering_procedure_(vall: torch.Tensor, handle: int, mg_filt: int) -> None:
    """filtering_procedure(mg_filt) on VALL in place (mgbf_filtering_procedure)."""
    _get(handle, MGBF).filtering_procedure(mg_filt, vall)


@filtering_procedure_.register_fake
def _(vall, handle, mg_filt):
    return None


@torch.library.custom_op("mgbf::filtering_procedure_adjoint_", mutates_args=("vall",))
def filtering_procedure_adjoint_(vall: torch.Tensor, handle: int, mg_filt: int) -> None:
    """The adjoint of filtering_procedure(mg_filt) on VALL in place."""
    _get(handle, MGBF).filtering_procedure_adjoint(mg_filt, vall)


@filtering_procedure_adjoint_.register_fake
def _(vall, handle, mg_filt):
    return None


@torch.library.custom_op("mgbf::batch_apply_", mutates_args=("fields",))
def batch_apply_(fields: List[torch.Tensor], batch: int, adjoint: bool) -> None:
    """One batched call over every variable group's field (mgbf_batch_apply)."""
    _get(batch, MGBFBatch).apply(list(fields), adjoint=adjoint)


@batch_apply_.register_fake
def _(fields, batch, adjoint):
    return None
