import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("het-scd_gb300", "oracle", "tests"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI of libscd_gb300.so)")


def pytest_terminal_summary(terminalreporter):
    import parity_log
    line = parity_log.summary()
    if line:
        terminalreporter.write_line(line)
