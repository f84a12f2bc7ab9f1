"""Stand-in for ``pytorch_lightning``, enough to construct the reference's
decoder module (CROMnet_secondary.NetDec) as a plain ``torch.nn.Module``.
Test infrastructure only; nothing trains through it."""
import torch


class LightningModule(torch.nn.Module):
    def save_hyperparameters(self, *a, **k):
        return None


class Trainer:
    def __init__(self, *a, **k):
        raise RuntimeError("training is not available in the test stand-in")


class Callback:
    pass
