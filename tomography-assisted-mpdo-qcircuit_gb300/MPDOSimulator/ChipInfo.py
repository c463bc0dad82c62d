"""Named chip presets (reference: MPDOSimulator/ChipInfo.py:8-98)."""


class ChipInformation:
    def __init__(self, query_time: str = None):
        self.queryTime = query_time
        self.status = None
        self.gateTime = None
        self.bath_rate = None
        self.dephasing_rate = None
        self.decay_rate = None
        self.T1 = None
        self.T2 = None
        self.chipName = None
        self.dpc_errorRate = None
        self.timeUnit = 'ns'

    def __getattr__(self, item):
        raise AttributeError(f'Chip: {item} is not supported.')

    def configure_chip(self, name: str, gate_time: float, decay_rate: float, dephasing_rate: float,
                       bath_rate: float, T1: float, T2: float, dpc_error_rate: float, status: bool):
        self.chipName = name
        self.gateTime = gate_time
        self.bath_rate = bath_rate
        self.decay_rate = decay_rate
        self.dephasing_rate = dephasing_rate
        self.T1 = T1
        self.T2 = T2
        self.dpc_errorRate = dpc_error_rate
        self.status = status

    def best(self):
        if self.queryTime is None:
            self.configure_chip('best', 30, 0.0, 0.0, 0., 2e11, 2e10, 11e-4, True)
        return self

    def medium(self):
        if self.queryTime is None:
            self.configure_chip('medium', 1, 0.98, 0.02, 0.01, 2e11, 2e10, 5e-2, True)
        return self

    def worst(self):
        if self.queryTime is None:
            self.configure_chip('worst', 30, 0.0, 0.0, 0., 2e2, 2e1, 11e-2, True)
        return self

    def show_property(self):
        """Print the chip's parameters, one per line."""
        rows = [('chip', self.chipName), ('gate time', f'{self.gateTime} {self.timeUnit}'),
                ('T1', f'{self.T1} {self.timeUnit}'), ('T2', f'{self.T2} {self.timeUnit}'),
                ('depolarising error rate', self.dpc_errorRate), ('status', self.status)]
        for name, value in rows:
            print(f'{name:>24}: {value}')
