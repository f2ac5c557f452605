"""Algorithmic HBM bytes of every kernel class of one predictor-corrector
step (each logical stage reads its inputs once and writes its outputs once).

N = nx*ny*nz points, Nh = (nx/2+1)*ny*nz half-spectrum points, s = bytes
of a real in the field precision (8 FP64, 4 FP32), complex = 2s.  Form-factor
tables are real (s per k-point).  The per-launch figure of a class is its
per-step bytes divided by its launches per step.
"""


def step_bytes(nx, ny, nz, otc=True, grad=True, s=8, renorm=True):
    N = nx * ny * nz
    Nh = (nx // 2 + 1) * ny * nz
    c = 2 * s
    b = {}
    # predictor: read psi, psiold3, hpsi1, hpsi2, pc, pot4, uimp;
    # write new psi (over psiold3), pc, hpsi2, den
    b["predict"] = (5 * c + 2 * s + 3 * c + s) * N
    # corrector: read psi, psiold3, psiold2, hpsi1, hpsi2, pc, pot4, uimp;
    # write pc, psi, den
    b["correct"] = (6 * c + 2 * s + 2 * c + s) * N
    # X1: read den, write its x-transformed half spectrum
    b["x1_r2c_den"] = s * N + c * Nh
    if grad:
        # first-derivative march: read den, write its three derivatives
        b["grad_march"] = 4 * s * N
    nconv1 = 3 if otc else 2
    nfwd2 = 4 if otc else 1
    # Y passes (in place): read + write each spectrum
    ny_arrays = 1 + nconv1 + nfwd2 + nfwd2 + (2 if otc else 0)
    b["fft_y_fwd"] = 2 * c * Nh * (1 + nfwd2 + (1 if otc else 0))
    b["fft_y_inv"] = 2 * c * Nh * (nconv1 + nfwd2 + (1 if otc else 0))
    assert ny_arrays * 2 * c * Nh == b["fft_y_fwd"] + b["fft_y_inv"]
    # Z passes with the k-space product: read input, per output read the
    # kernel table and write the product transform
    zc = (c * Nh + nconv1 * (s * Nh + c * Nh))
    zc += nfwd2 * (c * Nh + s * Nh + c * Nh)
    if otc:
        zc += c * Nh + s * Nh + c * Nh
    b["fft_z_conv"] = zc
    # X2: read the convolution spectra, den (+ grad den); write dencg, delj4,
    # pot4 (+ falfs) and the forward spectra
    b["x2_c2r_r2c"] = nconv1 * c * Nh + s * N + (3 * s * N if otc else 0) + (4 if otc else 3) * s * N + nfwd2 * c * Nh
    if otc:
        # X3: read 4 spectra, grad den, falfs, pot4; write pot4, I_xyz, g_y,
        # g_z, d(f I_x)/dx and the forward spectrum of grad(den).I
        b["x3_c2r_r2c"] = 4 * c * Nh + 5 * s * N + 7 * s * N + c * Nh
        # div march: read g_y, g_z; write dy g_y + dz g_z
        b["div_march"] = 3 * s * N
        # X4: read spectrum, den, dgx, dy g_y + dz g_z, pot4; write pot4, ualphas
        b["x4_c2r_ualpha"] = c * Nh + 4 * s * N + 2 * s * N
    else:
        b["x3_c2r_r2c"] = c * Nh + 2 * s * N + s * N
    if renorm:
        # an explicit rescale pass: psi and the history (psiold x3, hpsiold x2,
        # pc) read + written, den written.  The engines renormalise lazily
        # (per-buffer scale factors applied by the next step's kernels), so
        # their steps have no such pass.
        b["rescale"] = (14 * c + s) * N
    return b


def total_step_bytes(*a, **k):
    return sum(step_bytes(*a, **k).values())


def step_flops(nx, ny, nz, otc=True):
    """Algorithmic floating-point operations of one predictor-corrector step
    (FMA = 2), the count behind the FP64 ALU roofline:

    * real 3-D FFTs, 2.5 N log2 N each: 14 per OTC step (den forward; three
      convolution inverses; four forward, four inverse for the second-stage
      products; one forward, one inverse for div(f I)), 5 for OT;
    * two complex 13-point Laplacians (predictor, corrector): 3 axes x 13
      points of a real weight times a complex value, accumulated: 156 flop;
    * first-derivative stencils: grad den (3), d/dy and d/dz of f I (2) and
      the x-derivative of f I_x (1), 6 differences + 6 multiply-adds each =
      18 flop;
    * the k-space products (2 flop per half-spectrum point per table) and the
      point-wise algebra of the step (about 100 flop per point).
    """
    import math
    N = nx * ny * nz
    Nh = (nx // 2 + 1) * ny * nz
    nfft = 14 if otc else 5
    f = nfft * 2.5 * N * math.log2(N)
    f += 2 * 156 * N
    f += (6 if otc else 3) * 18 * N
    f += (8 if otc else 3) * 2 * Nh
    f += 100 * N
    return f
