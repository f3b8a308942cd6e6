"""The seeded synthetic workloads have the shapes and distributions the bench
lines state (no GPU): the periodic turbulence field (zero mean, rms 1, a
random-phase spectrum peaking where k^3 exp(-(k/10)^2) does, a periodic
halo), the dipole, the shear layer, the 96-instance ensemble and the served
request stream (Poisson arrivals at 40/s, 70 % Euler, sides and step counts
in their ranges)."""
import numpy as np

from fluid2d_gb300 import workloads as W

NH = 3


def test_turbulence_field():
    wl = W.turbulence(256, 256)
    w = wl["fields"]["vorticity"]
    assert w.shape == (256 + 2 * NH, 256 + 2 * NH)
    inner = w[NH:-NH, NH:-NH]
    assert abs(inner.mean()) < 1e-14 and abs(np.sqrt((inner ** 2).mean()) - 1) < 1e-12
    # the halo holds the periodic images
    assert np.array_equal(w[:NH, NH:-NH], inner[-NH:, :])
    assert np.array_equal(w[-NH:, NH:-NH], inner[:NH, :])
    assert np.array_equal(w[NH:-NH, :NH], inner[:, -NH:])
    assert np.array_equal(w[NH:-NH, -NH:], inner[:, :NH])
    # shell-summed spectrum: peak near sqrt(1.5) k0 = 12.2, negligible beyond 4 k0
    f = np.abs(np.fft.fft2(inner)) ** 2
    k = np.sqrt(np.add.outer(np.fft.fftfreq(256) ** 2, np.fft.fftfreq(256) ** 2)) * 256
    shells = np.bincount(np.rint(k).astype(int).ravel(), weights=f.ravel())
    smooth = np.convolve(shells, np.ones(5) / 5, mode="same")
    assert 9 <= int(np.argmax(smooth)) <= 16
    assert shells[50:].sum() < 1e-6 * shells.sum()
    assert shells[0] < 1e-20 * shells.sum()


def test_dipole_field():
    wl = W.dipole()
    w = wl["fields"]["vorticity"]
    xr, yr = W.cell_coords(128, 128, 1., 1.)
    jmax, imax = np.unravel_index(np.argmax(w), w.shape)
    jmin, imin = np.unravel_index(np.argmin(w), w.shape)
    assert abs(xr[jmax, imax] - 0.4) < 0.01 and abs(yr[jmax, imax] - 0.5) < 0.01
    assert abs(xr[jmin, imin] - 0.6) < 0.01 and abs(yr[jmin, imin] - 0.5) < 0.01
    assert np.all(w[wl["msk"] == 0] == 0)


def test_shear_layer():
    wl = W.shear()
    assert (wl["nx"], wl["ny"], wl["Lx"], wl["Ly"]) == (2048, 512, 4., 1.)
    w, b = wl["fields"]["vorticity"], wl["fields"]["buoyancy"]
    col = w[NH:-NH, 100]
    dy = 1. / 512
    # u = tanh((y - 1/2)/d): the column's vorticity integrates to u(1) - u(0) ~ 2 (w = -du/dy)
    assert abs(-col.sum() * dy - 2 * np.tanh(0.5 / 0.02)) < 1e-3
    assert np.abs(b[NH:-NH, NH:-NH]).max() < 1.01


def test_ensemble_members():
    ens = W.ensemble(96, seed=4)
    assert len(ens) == 96
    for wl in ens:
        assert wl["nx"] % 64 == 0 and wl["ny"] % 64 == 0
        assert 64 <= wl["nx"] <= 768 and 64 <= wl["ny"] <= 768
        assert abs(wl["Lx"] / wl["nx"] - wl["Ly"] / wl["ny"]) < 1e-15
        assert wl["msk"].shape == (wl["ny"] + 2 * NH, wl["nx"] + 2 * NH)
        assert np.all(wl["fields"]["vorticity"][wl["msk"] == 0] == 0)
    assert len({(wl["nx"], wl["ny"]) for wl in ens}) > 30


def test_served_stream():
    # the bench's sample: the first 200 of the 2000 requests (the stream's
    # draws are sequential, so a shorter stream is its prefix)
    count = 200
    st = W.served_stream(count)
    t = np.array([a for a, _, _ in st])
    assert len(st) == count and np.all(np.diff(t) > 0)
    assert abs(count / t[-1] - 40.) < 6.            # 2 sigma of a 200-arrival rate
    euler = np.mean([wl["model"] == "euler" for _, wl, _ in st])
    assert abs(euler - 0.7) < 0.07
    for _, wl, steps in st:
        assert 50 <= steps <= 500
        assert wl["nx"] % 128 == 0 and 128 <= wl["nx"] <= 2048
        assert wl["ny"] % 128 == 0 and 128 <= wl["ny"] <= 2048
        assert wl["msk"].shape == (wl["ny"] + 2 * NH, wl["nx"] + 2 * NH)
