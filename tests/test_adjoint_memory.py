"""The differentiable rollout's choice between keeping every step's stage
inputs and recomputing them from checkpoints (no GPU: the device-memory
query is replaced)."""
import pytest

torch = pytest.importorskip("torch")

from demon_simulation_code_gb300 import adjoint  # noqa: E402


class _Like:
    def __init__(self, n):
        self._n = n
        self.device = "cuda:0"

    def numel(self):
        return self._n


def test_stage_bytes_counts_sixteen_doubles_per_particle_and_step():
    assert adjoint.stage_bytes(200, 64 * 2048) == 200 * 16 * 64 * 2048 * 8  # 3.36 GB


@pytest.mark.parametrize("free, keep", [(80 << 30, True), (12 << 30, False), (16 << 30, True)])
def test_auto_keeps_the_stages_when_they_fit_a_quarter_of_free_memory(monkeypatch, free, keep):
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda device=None: (free, 280 << 30))
    need = adjoint.stage_bytes(200, 64 * 2048)
    assert (need <= free // 4) is keep
    assert adjoint._keep_all_stages("auto", 200, _Like(64 * 2048)) is keep


def test_auto_respects_the_byte_budget(monkeypatch):
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda device=None: (1 << 40, 1 << 40))
    steps = adjoint.STAGE_BUDGET_BYTES // (16 * 8 * 1000) + 1  # just over the budget
    assert adjoint._keep_all_stages("auto", steps, _Like(1000)) is False
    assert adjoint._keep_all_stages("auto", steps - 1, _Like(1000)) is True


def test_explicit_choices_and_bad_values(monkeypatch):
    def boom(device=None):
        raise AssertionError("no memory query for an explicit choice")

    monkeypatch.setattr(torch.cuda, "mem_get_info", boom)
    assert adjoint._keep_all_stages(True, 10, _Like(10)) is True
    assert adjoint._keep_all_stages(False, 10, _Like(10)) is False
    with pytest.raises(ValueError):
        adjoint._keep_all_stages("always", 10, _Like(10))
