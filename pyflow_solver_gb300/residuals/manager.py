"""Residual tracker, same contract as src/pyflow/residuals/manager.py:2-16.

Keeps the ``Ru`` series seeded with 1.0 (used by residual_drop_Ru_orders);
``plateau_detect`` always reports False, as in the reference.
"""


class ResidualManager:
    def __init__(self):
        class Series:
            def __init__(self):
                self.values = [1.0]
        self.series = {"Ru": Series()}

    def __call__(self, *args, **kwargs):
        return None

    def add(self, name, value):
        if name == "Ru":
            self.series["Ru"].values.append(value)

    def plateau_detect(self, name, window=10, threshold=-0.005):
        return False
