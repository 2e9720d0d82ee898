"""gen_FFT_PowerSpectra (simulations/Utilities/glow_up.py:752-827) for one column,
restated with numpy: max-normalise, |fft2|^2, radial bins from 1 - w/2 with
np.histogram, mean times annulus area; empty bins are 0 (the reference turns
them into NaN).  Test helper: the GPU spectrum is compared with it at sizes the
golden fixture does not hold, and it is itself pinned to the reference's output
(tests/test_oracle_pins.py)."""
import numpy as np


def spectrum_numpy(img, binwidth=0.5):
    L = img.shape[0]
    img = img.astype(np.float64)
    mx = img.max()
    img = img / (mx if mx != 0.0 else 1.0)
    kbins = np.arange(1 - binwidth / 2, L // 2 + 1, binwidth)
    kvals = 0.5 * (kbins[1:] + kbins[:-1])
    F = np.fft.fft2(img)
    kf = np.fft.fftfreq(L) * L
    kx, ky = np.meshgrid(kf, kf)
    knrm = np.sqrt(kx ** 2 + ky ** 2).flatten()
    amp = np.abs(F ** 2).flatten()
    s, _ = np.histogram(knrm, bins=kbins, weights=amp)
    c, _ = np.histogram(knrm, bins=kbins)
    p = np.divide(s, c, out=np.zeros_like(s), where=c != 0)
    p *= np.pi * (kbins[1:] ** 2 - kbins[:-1] ** 2)
    return kvals, p
