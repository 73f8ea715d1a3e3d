"""GPU drop-in for ``SingleProcessMediator`` (``mediator/single_process_mediator.py:57-156``): the configured run,
advanced as a batch of independent chains by the GPU engine.

A configuration switches to it by naming it in ``[Run]`` and giving its section the keys of
``[SingleProcessMediator]`` plus the batch options:

    [Run]
    mediator = gpu_chain_batch_mediator

    [GpuChainBatchMediator]
    state_handler = tree_state_handler
    scheduler = heap_scheduler
    activator = tag_activator
    input_output_handler = input_output_handler
    chains = 4096          ; independent chains (replicas of the configured initial state, own random numbers)
    mode = mixed           ; mixed (FP32 screening, FP64 re-solve) or exact (plain FP64)
    seed = 1

The factory builds the reference's objects exactly as for its own mediator (the constructor's annotations are the
reference's classes, from which the factory finds their packages); ``jellyfysh_gb300.plugin.plan`` turns them into
a batch of chains (atoms, or water molecules as composite objects) and runs it.  This module is imported by the
factory, with the reference present.
"""
from jellyfysh.activator import Activator
from jellyfysh.base.exceptions import EndOfRun
from jellyfysh.input_output_handler import InputOutputHandler
from jellyfysh.scheduler import Scheduler
from jellyfysh.state_handler import StateHandler

from jellyfysh_gb300.plugin.plan import run_plan, translate


class GpuChainBatchMediator:
    """The factory-built drop-in: same object graph as the reference's mediator, the run on the GPU."""

    def __init__(self, input_output_handler: InputOutputHandler, state_handler: StateHandler, scheduler: Scheduler,
                 activator: Activator, chains: int = 1, mode: str = "mixed", seed: int = 0,
                 events_per_launch: int = 256) -> None:
        from jellyfysh.setting import hypercubic_setting as setting
        state_handler.initialize(input_output_handler.read())
        self._input_output_handler = input_output_handler
        self.plan = translate(state_handler, activator, setting, chains, mode, seed, events_per_launch)
        self.batch = None

    def run(self) -> None:
        """Run every chain to the end-of-run time, then end the run as the reference does (EndOfRun)."""
        self.batch = run_plan(self.plan)
        raise EndOfRun("all chains reached the end-of-run time")

    def post_run(self) -> None:
        if self.batch is not None:
            self.batch.check_status()
