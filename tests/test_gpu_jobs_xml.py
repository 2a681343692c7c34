"""The reference's XML job files run end to end (LMultiSlice <action>, C# STEM
<Calculation_parameters>) and agree with the equivalent direct API calls."""
import numpy as np
import pytest

from multislice_gb300 import jobs, specimen as S
from multislice_gb300.mrc import read_mrc
from oracle import msl_oracle as O

pytestmark = pytest.mark.gpu

LMS = """<?xml version="1.0" ?>
<action>
    <io><fileNameInput>si.coo</fileNameInput><fileNameOutput>result/si_64</fileNameOutput></io>
    <image><nx>64</nx><ny>64</ny><dpa>6.0</dpa></image>
    <slicing><radiuc>20.0</radiuc><numberslices>8</numberslices></slicing>
    <microscope><aperture>25</aperture><cs>1.3</cs><defocus>-70</defocus><keV>200</keV></microscope>
</action>
"""

MUSLI = """<?xml version="1.0" encoding="utf-8" ?>
<Calculation_parameters>
  <ModelFileName>sto.coo</ModelFileName>
  <NSlices>2</NSlices>
  <atrad>3</atrad>
  <ThWaves><double>7.81</double><double>15.62</double></ThWaves>
  <N>128</N><M>128</M>
  <E><double>200000</double></E>
  <IniWaveType>STEMshift</IniWaveType>
  <BeamShift>
    <ArrayOfDouble><double>3</double><double>2</double></ArrayOfDouble>
    <ArrayOfDouble><double>0.1</double><double>0.2</double></ArrayOfDouble>
    <ArrayOfDouble><double>0.7</double><double>0.6</double></ArrayOfDouble>
  </BeamShift>
  <ConvAngles><ArrayOfDouble><double>0.9</double><double>0.0</double></ArrayOfDouble></ConvAngles>
  <DetectorAngles>
    <ArrayOfDouble><double>7.9</double><double>3.2</double></ArrayOfDouble>
    <ArrayOfDouble><double>0.88</double><double>0.44</double></ArrayOfDouble>
  </DetectorAngles>
  <Df><double>0</double></Df><Cs><double>0</double></Cs>
</Calculation_parameters>
"""


def test_lmultislice_action_job(tmp_path, ctx):
    spec = S.si_diamond(2, 2, 2)
    S.write_coo(spec, str(tmp_path / "si.coo"))
    (tmp_path / "result").mkdir()
    (tmp_path / "job.xml").write_text(LMS)
    res = jobs.run_job_file(str(tmp_path / "job.xml"))
    v, _ = read_mrc(res["potential"])
    img, _ = read_mrc(res["image"])
    back = S.read_coo(str(tmp_path / "si.coo"))
    vv = ctx.potential(back, 64, 64, 8, res["radius"])
    assert np.array_equal(v, vv)
    t = ctx.transmission(vv, back.ax, back.by, 200.0)
    k_obj = 25e-3 / O.wavelength(200.0)
    ref, _, _ = ctx.ctem_image(t, back.cz / 8, np.arange(8), back.ax, back.by, 200.0, 1.3e7, -700.0, k_obj)
    assert O.rel_l2(img[0], ref) < 1e-6


def test_musli_stemshift_job(tmp_path, ctx):
    spec = S.srtio3(2, 2, 1)
    S.write_coo(spec, str(tmp_path / "sto.coo"))
    (tmp_path / "job.xml").write_text(MUSLI)
    res = jobs.run_job_file(str(tmp_path / "job.xml"))
    img = res["stem"]
    assert img.shape == (3, 2, 2, 2) and res["checkpoints"] == [3, 7]
    back = S.read_coo(str(tmp_path / "sto.coo"))
    v = ctx.potential(back, 128, 128, 2, 3.0)
    t = ctx.transmission(v, back.ax, back.by, 200.0)
    xy = S.raster(0.1 * back.ax, 0.7 * back.ax, 0.2 * back.by, 0.6 * back.by, 3, 2)
    d = ctx.stem_scan(t, back.cz / 2, np.arange(8) % 2, back.ax, back.by, 200.0, 0.9, xy,
                      [(3.2, 7.9), (0.44, 0.88)], checkpoints=[3, 7])
    assert np.array_equal(d.reshape(3, 2, 2, 2), img)
    f, _ = read_mrc(str(tmp_path / "sto_stem_15.62A_det0.mrc"))
    assert np.allclose(f[0], img[:, :, 1, 0])


MUSLI_PW = """<?xml version="1.0" encoding="utf-8" ?>
<Calculation_parameters>
  <ModelFileName>sto.coo</ModelFileName>
  <NSlices>2</NSlices>
  <SaveSlices>true</SaveSlices>
  <IsSaveDiffractions>true</IsSaveDiffractions>
  <atrad>3</atrad>
  <ThWaves><double>7.81</double></ThWaves>
  <N>128</N><M>128</M>
  <E><double>200000</double></E>
  <IniWaveType>PlaneWave</IniWaveType>
</Calculation_parameters>
"""


def test_musli_planewave_job_writes_csharp_files(tmp_path, ctx):
    from multislice_gb300 import csfiles as C
    spec = S.srtio3(2, 2, 1)
    S.write_coo(spec, str(tmp_path / "sto.coo"))
    (tmp_path / "job.xml").write_text(MUSLI_PW)
    res = jobs.run_job_file(str(tmp_path / "job.xml"))
    back = S.read_coo(str(tmp_path / "sto.coo"))
    v = ctx.potential(back, 128, 128, 2, 3.0)
    t = ctx.transmission(v, back.ax, back.by, 200.0)
    w = ctx.multislice(t, back.cz / 2, np.arange(4) % 2, back.ax, back.by, 200.0)[0]
    wav, meta = C.read_wav(str(tmp_path / "sto_wave_7.81A.wav"))
    assert np.array_equal(wav, w.astype(np.complex128)) and res["checkpoints"] == [3]
    cbed, _ = C.read_cbed(str(tmp_path / "sto_diffraction_7.81A.cbed"))
    ref = O.kfft(w.astype(np.complex128)[None])[0]
    assert O.rel_l2(cbed, np.abs(ref) ** 2) < 1e-5
    assert abs(cbed.sum() - (128 * 128) ** 2 * np.mean(np.abs(w) ** 2)) < 1e-4 * cbed.sum()   # Parseval
    sl, meta = C.read_slice(str(tmp_path / "Slice stack" / "Slice_0001.slice"))
    assert np.array_equal(sl, t[1].astype(np.complex128)) and meta["f9"] == 1 and meta["f10"] == 2


def test_kirkland_mulslice_from_tiff_layers(tmp_path, ctx):
    """Layer potentials as floatTIFF files (vz with phase lambda mm0 vz) and a
    stacking sequence -> exit wave TIFF, against the direct library calls."""
    from multislice_gb300 import floattiff as FT, kirkland as K
    spec = S.si_diamond(2, 2, 1)
    v = ctx.potential(spec, 64, 64, 2, 3.0)
    kev = 200.0
    f32 = np.float32
    scale = f32(f32(O.wavelength(kev)) * (f32(1.0) + f32(kev) / f32(511.0)))
    files = []
    for i in range(2):
        vz = (v[i].astype(np.float64) * O.sigma(kev) / float(scale)).astype(np.float32)
        par = np.zeros(512, np.float32)
        par[FT.P["C"]] = spec.cz / 2
        par[FT.P["DX"]], par[FT.P["DY"]] = spec.ax / 64, spec.by / 64
        FT.write_float_tiff(tmp_path / f"l{i}.tif", vz, params=par, dx=spec.ax / 64, dy=spec.by / 64)
        files.append(str(tmp_path / f"l{i}.tif"))
    w, seq = K.mulslice(ctx, files, "6(ab)", kev, str(tmp_path / "w.tif"))
    assert seq == [0, 1] * 6
    back, par = FT.read_exit_wave(str(tmp_path / "w.tif"))
    assert np.array_equal(back, w) and par[FT.P["NSLICES"]] == 12
    t = ctx.transmission(v, spec.ax, spec.by, kev)
    ref = ctx.multislice(t, spec.cz / 2, seq, spec.ax, spec.by, kev)[0]
    assert O.rel_l2(back, ref) < 2e-6


def _musli_job(kind, ths, extra=""):
    return f"""<?xml version="1.0" encoding="utf-8" ?>
<Calculation_parameters>
  <ModelFileName>sto.coo</ModelFileName>
  <NSlices>2</NSlices>
  <atrad>3</atrad>
  <ThWaves>{''.join(f'<double>{t}</double>' for t in ths)}</ThWaves>
  <N>128</N><M>128</M>
  <E><double>200000</double></E>
  <IniWaveType>{kind}</IniWaveType>{extra}
</Calculation_parameters>
"""


def test_musli_precalculated_wave_resumes_the_run(tmp_path, ctx):
    """Checkpoint / resume: a run stopped at 7.81 A and continued from its .wav
    equals the uninterrupted run to 15.62 A (MSProject.cs:423-440)."""
    from multislice_gb300 import csfiles as C
    S.write_coo(S.srtio3(2, 2, 2), str(tmp_path / "sto.coo"))
    ax = S.read_coo(str(tmp_path / "sto.coo")).ax
    (tmp_path / "a.xml").write_text(_musli_job("PlaneWave", [7.81]))
    jobs.run_job_file(str(tmp_path / "a.xml"))
    (tmp_path / "b.xml").write_text(_musli_job("Precalculated", [15.62],
                                               "\n  <IniWaveFileName>sto_wave_7.81A.wav</IniWaveFileName>"))
    resumed = jobs.run_job_file(str(tmp_path / "b.xml"))["waves"][0]
    (tmp_path / "c.xml").write_text(_musli_job("PlaneWave", [15.62]))
    whole = jobs.run_job_file(str(tmp_path / "c.xml"))["waves"][0]
    assert O.rel_l2(resumed, whole) < 1e-6
    _, meta = C.read_wav(str(tmp_path / "sto_wave_15.62A.wav"))
    assert meta["f9"] == 15.62
    # a start wave on another grid is refused before any work
    C.write_wav(str(tmp_path / "bad.wav"), np.ones((64, 64), np.complex64), ax, ax, 7.81, 200.0)
    (tmp_path / "d.xml").write_text(_musli_job("Precalculated", [15.62],
                                               "\n  <IniWaveFileName>bad.wav</IniWaveFileName>"))
    with pytest.raises(ValueError):
        jobs.run_job_file(str(tmp_path / "d.xml"))
