"""GB300 twin of ``tensorf/utils.py``."""
import math


def psnr_from_mse(mse: float) -> float:
    """utils.py:4-9: -10 log10(max(mse, 1e-10))."""
    return -10.0 * math.log10(max(float(mse), 1e-10))
