"""The fitting loop's control flow (``training.fit``) with a stand-in for the GPU step: the scheduler is
stepped with every epoch's loss, the best model is kept and written, batches are seeded subsets, and the
loop stops after ``early_stopping_patience`` epochs without improvement."""
import json
import os

import numpy as np
import torch

from slakonet_gb300 import model as M, synthetic as syn, training as T


def test_fit_keeps_the_best_model_and_stops_early(tmp_path, monkeypatch):
    zs = [6]
    sd = syn.default_shell_dict()
    model = M.MultiElementSkfParameterOptimizer.from_tables(syn.make_tables(zs, {6: sd[6]}, seed=2))
    losses = iter([5.0, 4.0, 3.0, 3.5, 3.6, 3.7, 3.8, 3.9, 9.0, 9.0])
    seen = []

    def fake_step(model_, optimizer, structures, dos_t, gap_t, shell_dict, device, scheduler=None):
        seen.append(len(structures))
        with torch.no_grad():
            for p in model_.parameters():
                p.add_(1.0)                      # every epoch moves the parameters
        loss = next(losses)
        scheduler.step(loss)
        return {"loss": loss, "structures_used": len(structures)}
    monkeypatch.setattr(T, "train_step", fake_step)
    sts = [{"numbers": [6], "positions": [[0.0, 0.0, 0.0]], "cell": np.eye(3) * 8.0, "kpoints": [[0.0, 0.0, 0.0]]}
           for _ in range(6)]
    before = {k: v.clone() for k, v in model.state_dict().items()}
    out = T.fit(model, sts, torch.zeros(6, 1000), torch.zeros(6), sd, "cpu", num_epochs=50, batch_size=4,
                save_directory=str(tmp_path), early_stopping_patience=5)
    assert [h["loss"] for h in out["history"]] == [5.0, 4.0, 3.0, 3.5, 3.6, 3.7, 3.8, 3.9]   # 5 after the best
    assert out["best_loss"] == 3.0 and out["best_epoch"] == 2 and seen == [4] * 8
    k = next(iter(before))

    def after(epochs):                           # the parameters after that many of the stand-in's steps
        t = before[k].clone()
        for _ in range(epochs):
            t += 1.0
        return t
    assert torch.equal(out["best_state"][k], after(3))                                  # the state after epoch 2
    best = M.MultiElementSkfParameterOptimizer.load_ultra_compact(os.path.join(tmp_path, "best_model.pt"))
    assert torch.equal(best.state_dict()[k], after(3))
    final = M.MultiElementSkfParameterOptimizer.load_ultra_compact(os.path.join(tmp_path, "final_model.pt"))
    assert torch.equal(final.state_dict()[k], after(8))
    hist = json.load(open(os.path.join(tmp_path, "training_history.json")))
    assert hist["best_epoch"] == 2 and len(hist["history"]) == 8
