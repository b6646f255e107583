// Host-side check of the FP64 fast-path math in sse_device.cuh against the
// reference's formulas (ConservationLaws.jl:132-156,
// euler_navierstokes.jl:100-131, 171-195), on seeded random states.
// Built and run by tests/test_device_math.py with nvcc; needs no GPU.
#include <cmath>
#include <cstdio>
#include <random>

#include "../cloud.jl_gb300/csrc/sse_device.cuh"

using namespace sse;

static double ref_logmean(double x, double y) {
  double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4) return (x + y) * 105 / (210 + f2 * (70 + f2 * (42 + f2 * 30)));
  return (y - x) / std::log(y / x);
}
static double ref_inv_logmean(double x, double y) {
  double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4) return (210 + f2 * (70 + f2 * (42 + f2 * 30))) / ((x + y) * 105);
  return std::log(y / x) / (y - x);
}

template <int D>
static void ref_ec_tensor(double g, const double *uL, const double *uR, double F[D + 2][D]) {
  const double gm1 = g - 1, igm1 = 1 / (g - 1);
  double VL[D], VR[D], sL = 0, sR = 0, vv = 0;
  for (int m = 0; m < D; ++m) { VL[m] = uL[m + 1] / uL[0]; VR[m] = uR[m + 1] / uR[0]; }
  for (int m = 0; m < D; ++m) { sL += VL[m] * VL[m]; sR += VR[m] * VR[m]; vv += VL[m] * VR[m]; }
  double pL = gm1 * (uL[D + 1] - 0.5 * uL[0] * sL), pR = gm1 * (uR[D + 1] - 0.5 * uR[0] * sR);
  double rho = ref_logmean(uL[0], uR[0]), pavg = 0.5 * (pL + pR);
  double C = 0.5 * vv + igm1 * ref_inv_logmean(uL[0] / pL, uR[0] / pR);
  for (int n = 0; n < D; ++n) {
    double va = 0.5 * (VL[n] + VR[n]);
    F[0][n] = rho * va;
    for (int m = 0; m < D; ++m) F[m + 1][n] = rho * 0.5 * (VL[m] + VR[m]) * va + (m == n ? pavg : 0);
    F[D + 1][n] = rho * va * C + 0.5 * (pL * VR[n] + pR * VL[n]);
  }
}

template <int D>
static void ref_c2e(double g, const double *u, double *w) {
  double s = 0;
  for (int m = 0; m < D; ++m) s += u[m + 1] * u[m + 1];
  double k = (0.5 / u[0]) * s, p = (g - 1) * (u[D + 1] - k), ip = 1 / p;
  w[0] = (g - std::log(p / std::pow(u[0], g))) / (g - 1) - k * ip;
  for (int m = 0; m < D; ++m) w[m + 1] = u[m + 1] * ip;
  w[D + 1] = -u[0] * ip;
}

template <int D>
static void ref_e2c(double g, const double *wi, double *u) {
  double w[D + 2], s = 0;
  for (int e = 0; e < D + 2; ++e) w[e] = wi[e] * (g - 1);
  for (int m = 0; m < D; ++m) s += w[m + 1] * w[m + 1];
  double k = s / (2 * w[D + 1]), sv = g - w[0] + k;
  double rhoe = std::pow((g - 1) / std::pow(-w[D + 1], g), 1 / (g - 1)) * std::exp(-sv / (g - 1));
  u[0] = -w[D + 1] * rhoe;
  for (int m = 0; m < D; ++m) u[m + 1] = w[m + 1] * rhoe;
  u[D + 1] = rhoe * (1 - k);
}

template <int D>
static void random_state(std::mt19937_64 &rng, double g, double pscale, double *u) {
  std::uniform_real_distribution<double> U(-1, 1);
  double rho = 1.0 + 0.3 * U(rng), p = pscale * (1.0 + 0.3 * U(rng)), ke = 0;
  u[0] = rho;
  for (int m = 0; m < D; ++m) { double v = U(rng); u[m + 1] = rho * v; ke += 0.5 * rho * v * v; }
  u[D + 1] = p / (g - 1) + ke;
}

static double rel(double a, double b) { return std::fabs(a - b) / std::fmax(std::fabs(b), 1e-300); }

template <int D>
static void check(std::mt19937_64 &rng, double *worst) {
  const double g = 1.4;
  std::uniform_real_distribution<double> U(-1, 1);
  for (int trial = 0; trial < 20000; ++trial) {
    double pscale = (trial % 2) ? 71.4 : 1.0;
    double uL[D + 2], uR[D + 2];
    random_state<D>(rng, g, pscale, uL);
    // near pairs (series branch) and far pairs (log branch)
    if (trial % 3) {
      for (int e = 0; e < D + 2; ++e) uR[e] = uL[e] * (1.0 + 1e-3 * U(rng));
    } else {
      random_state<D>(rng, g, pscale, uR);
    }
    double x = uL[0], y = uR[0];
    worst[0] = std::fmax(worst[0], rel(logmean_fast(x, y), ref_logmean(x, y)));
    worst[1] = std::fmax(worst[1], rel(inv_logmean_fast(x, y), ref_inv_logmean(x, y)));
    double PL[3 + D], PR[3 + D], G[D];
    euler_prim_fast<D>(g - 1, uL, PL);
    euler_prim_fast<D>(g - 1, uR, PR);
    for (int m = 0; m < D; ++m) G[m] = U(rng);
    double out[D + 2], F[D + 2][D];
    ec_flux_dot<D>(1 / (g - 1), PL, PR, G, out);
    {
      // the halved-vector form reproduces ec_flux_dot's mass and momentum
      // fluxes bit for bit and its energy flux to rounding
      double Gh[D], oh[D + 2];
      const double ig = 1 / (g - 1);
      const double q[4] = {ig * 2.0, ig * (2.0 / 3.0), ig * 0.4, ig * (2.0 / 7.0)};
      for (int m = 0; m < D; ++m) Gh[m] = 0.5 * G[m];
      ec_flux_dot_half<D>(ig, q, PL, PR, Gh, oh);
      for (int e = 0; e < D + 1; ++e)
        if (oh[e] != out[e]) worst[10] += 1.0;
      double escale = 0;
      for (int e = 0; e < D + 2; ++e) escale = std::fmax(escale, std::fabs(out[e]));
      worst[15] = std::fmax(worst[15], std::fabs(oh[D + 1] - out[D + 1]) / escale);
    }
    ref_ec_tensor<D>(g, uL, uR, F);
    double scale = 0;
    for (int e = 0; e < D + 2; ++e)
      for (int n = 0; n < D; ++n) scale = std::fmax(scale, std::fabs(F[e][n]));
    for (int e = 0; e < D + 2; ++e) {
      double want = 0;
      for (int n = 0; n < D; ++n) want += G[n] * F[e][n];
      worst[2] = std::fmax(worst[2], std::fabs(out[e] - want) / scale);
    }
    double w1[D + 2], w2[D + 2], u1[D + 2], u2[D + 2];
    cons_to_entropy_fast<D>(g, g - 1, 1 / (g - 1), uL, w1);
    ref_c2e<D>(g, uL, w2);
    for (int e = 0; e < D + 2; ++e) worst[3] = std::fmax(worst[3], rel(w1[e], w2[e]));
    entropy_to_cons_fast<D>(g, g - 1, 1 / (g - 1), std::log(g - 1), w2, u1);
    ref_e2c<D>(g, w2, u2);
    for (int e = 0; e < D + 2; ++e) worst[4] = std::fmax(worst[4], std::fabs(u1[e] - u2[e]) / std::fabs(u2[D + 1]));
  }
}

// Mixed form: FP32 contracted flux on perturbations from a reference state,
// with the momentum flux reduced by p_ref and the energy flux by H_ref f_rho,
// against the FP64 contracted flux; errors are relative to the size of the
// reduced flux components (what the FP32 arithmetic has to resolve).
template <int D>
static void check_mixed(std::mt19937_64 &rng, double *worst) {
  const double g = 1.4, gm1 = g - 1;
  std::uniform_real_distribution<double> U(-1, 1);
  const double rho_ref = 1.0, E_ref = 71.4 / gm1 + 0.3, p_ref = gm1 * E_ref;
  const double theta_ref = p_ref / rho_ref, H_ref = g / gm1 * theta_ref;
  for (int trial = 0; trial < 20000; ++trial) {
    // low-Mach states: unit-size velocity and density variation, pressure
    // 71.4 with 1 % fluctuations; neighbours within 0.1 % or 20 %
    double uL[D + 2], uR[D + 2];
    {
      double rho = 1.0 + 0.3 * U(rng), p = 71.4 * (1.0 + 0.01 * U(rng)), ke = 0;
      uL[0] = rho;
      for (int m = 0; m < D; ++m) { double v = U(rng); uL[m + 1] = rho * v; ke += 0.5 * rho * v * v; }
      uL[D + 1] = p / gm1 + ke;
    }
    for (int e = 0; e < D + 2; ++e) uR[e] = uL[e] * (1.0 + ((trial % 4) ? 1e-3 : 2e-1) * U(rng));
    double PL[3 + D], PR[3 + D], G[D], out[D + 2];
    euler_prim_fast<D>(gm1, uL, PL);
    euler_prim_fast<D>(gm1, uR, PR);
    for (int m = 0; m < D; ++m) G[m] = U(rng);
    ec_flux_dot<D>(1 / gm1, PL, PR, G, out);
    // reduced FP64 reference values
    double want[D + 2];
    for (int e = 0; e < D + 2; ++e) want[e] = out[e];
    for (int m = 0; m < D; ++m) want[1 + m] -= p_ref * G[m];
    want[D + 1] -= H_ref * out[0];
    float dL[D + 2], dR[D + 2], QL[4 + D], QR[4 + D], Gf[D], got[D + 2];
    for (int e = 0; e < D + 2; ++e) {
      double ref = (e == 0) ? rho_ref : (e == D + 1 ? E_ref : 0.0);
      dL[e] = (float)(uL[e] - ref);
      dR[e] = (float)(uR[e] - ref);
    }
    for (int m = 0; m < D; ++m) Gf[m] = (float)G[m];
    euler_prim_mixed<D>((float)gm1, (float)rho_ref, (float)p_ref, dL, QL);
    euler_prim_mixed<D>((float)gm1, (float)rho_ref, (float)p_ref, dR, QR);
    ec_flux_dot_mixed<D>((float)(1 / gm1), (float)rho_ref, (float)theta_ref, QL, QR, Gf, got);
    double scale = 0;
    for (int e = 0; e < D + 2; ++e) scale = std::fmax(scale, std::fabs(want[e]));
    for (int e = 0; e < D + 2; ++e) worst[5] = std::fmax(worst[5], std::fabs(got[e] - want[e]) / scale);
  }
}

// Reverse-mode functions against central differences of the forward ones
// (relative errors of O(h^2) + O(eps/h), h = 1e-6 relative).
template <int D>
static void check_adjoint(std::mt19937_64 &rng, double *worst) {
  const double g = 1.4, gm1 = g - 1, igm1 = 1 / gm1;
  std::uniform_real_distribution<double> U(-1, 1);
  for (int trial = 0; trial < 2000; ++trial) {
    double pscale = (trial % 2) ? 71.4 : 1.0;
    double uL[D + 2], uR[D + 2];
    random_state<D>(rng, g, pscale, uL);
    if (trial % 3) {
      for (int e = 0; e < D + 2; ++e) uR[e] = uL[e] * (1.0 + 1e-3 * U(rng));
    } else {
      random_state<D>(rng, g, pscale, uR);
    }
    double G[D], ob[D + 2], du[D + 2];
    for (int m = 0; m < D; ++m) G[m] = U(rng);
    for (int e = 0; e < D + 2; ++e) { ob[e] = U(rng); du[e] = U(rng); }
    // flux: d/du_L of ob . ECdot(prim(uL), prim(uR), G) via prims
    double PL[3 + D], PR[3 + D], PbL[3 + D], PbR[3 + D], ubL[D + 2] = {0}, ubR[D + 2] = {0};
    euler_prim_fast<D>(gm1, uL, PL);
    euler_prim_fast<D>(gm1, uR, PR);
    ec_flux_dot_bwd<D>(igm1, PL, PR, G, ob, PbL, PbR);
    euler_prim_bwd<D>(gm1, uL, PL, PbL, ubL);
    euler_prim_bwd<D>(gm1, uR, PR, PbR, ubR);
    auto J = [&](const double *a, const double *b) {
      double Pa[3 + D], Pb_[3 + D], o[D + 2], s = 0;
      euler_prim_fast<D>(gm1, a, Pa);
      euler_prim_fast<D>(gm1, b, Pb_);
      ec_flux_dot<D>(igm1, Pa, Pb_, G, o);
      for (int e = 0; e < D + 2; ++e) s += ob[e] * o[e];
      return s;
    };
    double sL = 0, sR = 0, dirL = 0, dirR = 0;
    double h = 1e-6;
    double a1[D + 2], a2[D + 2], b1[D + 2], b2[D + 2];
    for (int e = 0; e < D + 2; ++e) {
      double he = h * std::fabs(uL[e]) + 1e-9;
      a1[e] = uL[e] + he * du[e]; a2[e] = uL[e] - he * du[e];
      sL += ubL[e] * du[e] * he;
      double hr = h * std::fabs(uR[e]) + 1e-9;
      b1[e] = uR[e] + hr * du[e]; b2[e] = uR[e] - hr * du[e];
      sR += ubR[e] * du[e] * hr;
    }
    dirL = 0.5 * (J(a1, uR) - J(a2, uR));
    dirR = 0.5 * (J(uL, b1) - J(uL, b2));
    // floor: the round-off of the central difference itself, |J| eps / h
    double scaleL = std::fabs(sL) + 1e-10 * std::fabs(J(uL, uR)) * h;
    double scaleR = std::fabs(sR) + 1e-10 * std::fabs(J(uL, uR)) * h;
    worst[6] = std::fmax(worst[6], std::fabs(dirL - sL) / scaleL);
    worst[6] = std::fmax(worst[6], std::fabs(dirR - sR) / scaleR);
    // entropy maps: JVP against central differences, and Jacobian symmetry
    double w[D + 2], jw[D + 2], wp[D + 2], wm[D + 2], up[D + 2], um[D + 2];
    cons_to_entropy_fast<D>(g, gm1, igm1, uL, w);
    cons_to_entropy_jvp<D>(g, gm1, igm1, uL, du, jw);
    for (int e = 0; e < D + 2; ++e) { up[e] = uL[e] + h * du[e]; um[e] = uL[e] - h * du[e]; }
    cons_to_entropy_fast<D>(g, gm1, igm1, up, wp);
    cons_to_entropy_fast<D>(g, gm1, igm1, um, wm);
    double nrm = 0;
    for (int e = 0; e < D + 2; ++e) nrm = std::fmax(nrm, std::fabs(jw[e]));
    for (int e = 0; e < D + 2; ++e)
      worst[7] = std::fmax(worst[7], std::fabs((wp[e] - wm[e]) / (2 * h) - jw[e]) / nrm);
    double ju[D + 2];
    entropy_to_cons_jvp<D>(g, gm1, igm1, std::log(gm1), w, du, ju);
    double wpp[D + 2], wmm[D + 2], uu1[D + 2], uu2[D + 2];
    double hw = 1e-7;
    for (int e = 0; e < D + 2; ++e) { wpp[e] = w[e] + hw * du[e]; wmm[e] = w[e] - hw * du[e]; }
    entropy_to_cons_fast<D>(g, gm1, igm1, std::log(gm1), wpp, uu1);
    entropy_to_cons_fast<D>(g, gm1, igm1, std::log(gm1), wmm, uu2);
    nrm = 0;
    for (int e = 0; e < D + 2; ++e) nrm = std::fmax(nrm, std::fabs(ju[e]));
    for (int e = 0; e < D + 2; ++e)
      worst[7] = std::fmax(worst[7], std::fabs((uu1[e] - uu2[e]) / (2 * hw) - ju[e]) / nrm);
    // symmetry: a . J b == b . J a
    double a[D + 2], b[D + 2], Ja[D + 2], Jb[D + 2];
    for (int e = 0; e < D + 2; ++e) { a[e] = U(rng); b[e] = U(rng); }
    cons_to_entropy_jvp<D>(g, gm1, igm1, uL, a, Ja);
    cons_to_entropy_jvp<D>(g, gm1, igm1, uL, b, Jb);
    double x1 = 0, x2 = 0, sc = 0;
    for (int e = 0; e < D + 2; ++e) { x1 += b[e] * Ja[e]; x2 += a[e] * Jb[e]; sc += std::fabs(b[e] * Ja[e]); }
    worst[8] = std::fmax(worst[8], std::fabs(x1 - x2) / sc);
    entropy_to_cons_jvp<D>(g, gm1, igm1, std::log(gm1), w, a, Ja);
    entropy_to_cons_jvp<D>(g, gm1, igm1, std::log(gm1), w, b, Jb);
    x1 = x2 = sc = 0;
    for (int e = 0; e < D + 2; ++e) { x1 += b[e] * Ja[e]; x2 += a[e] * Jb[e]; sc += std::fabs(b[e] * Ja[e]); }
    worst[8] = std::fmax(worst[8], std::fabs(x1 - x2) / sc);
  }
}

// Mixed-form reverse mode: the FP32 transpose of the reduced flux with the
// transformed cotangent (ob_rho + H_ref ob_E, ob_m, ob_E), mapped to
// conservative-perturbation cotangents, against the FP64 transpose of the
// full flux mapped to conservative cotangents (the same quantity); errors
// relative to the largest FP64 cotangent of the pair.
template <int D>
static void check_mixed_adjoint(std::mt19937_64 &rng, double *worst) {
  const double g = 1.4, gm1 = g - 1;
  std::uniform_real_distribution<double> U(-1, 1);
  const double rho_ref = 1.0, E_ref = 71.4 / gm1 + 0.3, p_ref = gm1 * E_ref;
  const double theta_ref = p_ref / rho_ref, H_ref = g / gm1 * theta_ref;
  for (int trial = 0; trial < 20000; ++trial) {
    double uL[D + 2], uR[D + 2];
    {
      double rho = 1.0 + 0.3 * U(rng), p = 71.4 * (1.0 + 0.01 * U(rng)), ke = 0;
      uL[0] = rho;
      for (int m = 0; m < D; ++m) { double v = U(rng); uL[m + 1] = rho * v; ke += 0.5 * rho * v * v; }
      uL[D + 1] = p / gm1 + ke;
    }
    for (int e = 0; e < D + 2; ++e) uR[e] = uL[e] * (1.0 + ((trial % 4) ? 1e-3 : 2e-1) * U(rng));
    double PL[3 + D], PR[3 + D], G[D], ob[D + 2], PbL[3 + D], PbR[3 + D];
    euler_prim_fast<D>(gm1, uL, PL);
    euler_prim_fast<D>(gm1, uR, PR);
    for (int m = 0; m < D; ++m) G[m] = U(rng);
    for (int e = 0; e < D + 2; ++e) ob[e] = U(rng);
    ec_flux_dot_bwd<D>(1 / gm1, PL, PR, G, ob, PbL, PbR);
    double ubL[D + 2] = {0}, ubR[D + 2] = {0};
    euler_prim_bwd<D>(gm1, uL, PL, PbL, ubL);
    euler_prim_bwd<D>(gm1, uR, PR, PbR, ubR);
    float dL[D + 2], dR[D + 2], QL[4 + D], QR[4 + D], Gf[D], obf[D + 2], QbL[4 + D], QbR[4 + D];
    for (int e = 0; e < D + 2; ++e) {
      double ref = (e == 0) ? rho_ref : (e == D + 1 ? E_ref : 0.0);
      dL[e] = (float)(uL[e] - ref);
      dR[e] = (float)(uR[e] - ref);
      obf[e] = (float)ob[e];
    }
    obf[0] = (float)(ob[0] + H_ref * ob[D + 1]);
    for (int m = 0; m < D; ++m) Gf[m] = (float)G[m];
    euler_prim_mixed<D>((float)gm1, (float)rho_ref, (float)p_ref, dL, QL);
    euler_prim_mixed<D>((float)gm1, (float)rho_ref, (float)p_ref, dR, QR);
    ec_flux_dot_mixed_bwd<D>((float)(1 / gm1), (float)rho_ref, (float)theta_ref, QL, QR, Gf, obf, QbL, QbR);
    float vbL[D + 2] = {0}, vbR[D + 2] = {0};
    euler_prim_mixed_bwd<D>((float)gm1, (float)theta_ref, QL, QbL, vbL);
    euler_prim_mixed_bwd<D>((float)gm1, (float)theta_ref, QR, QbR, vbR);
    double scale = 0;
    for (int e = 0; e < D + 2; ++e) scale = std::fmax(scale, std::fmax(std::fabs(ubL[e]), std::fabs(ubR[e])));
    for (int e = 0; e < D + 2; ++e) {
      worst[9] = std::fmax(worst[9], std::fabs(vbL[e] - ubL[e]) / scale);
      worst[9] = std::fmax(worst[9], std::fabs(vbR[e] - ubR[e]) / scale);
    }
  }
}

// FP32 perturbation entropy maps of the mixed form's phase A against the
// FP64 maps: dw = w(u_ref + du) - w_ref and du = u(w_ref + dw) - u_ref, with
// the FP32 inputs taken exactly, relative to the largest component of the
// perturbation.  Low-Mach states (pressure 71.4, unit velocities) with
// density and pressure perturbations of 0.1 %, 3 % and 30 %.
template <int D>
static void check_entropy_pert(std::mt19937_64 &rng, double *worst) {
  const double g = 1.4, gm1 = g - 1, igm1 = 1 / gm1, lg = std::log(gm1);
  std::uniform_real_distribution<double> U(-1, 1);
  Physics ph{};
  ph.gamma = g; ph.gm1 = gm1; ph.igm1 = igm1;
  ph.rho_ref = 1.0; ph.E_ref = 71.4 / gm1; ph.p_ref = gm1 * ph.E_ref;
  double uref[D + 2] = {};
  uref[0] = ph.rho_ref;
  uref[D + 1] = ph.E_ref;
  cons_to_entropy_fast<D>(g, gm1, igm1, uref, ph.w_ref);
  ph.ip_ref = 1 / ph.p_ref;
  ph.irho_ref = 1 / ph.rho_ref;
  ph.a_ref = -gm1 * ph.w_ref[D + 1];
  ph.ia_ref = 1 / ph.a_ref;
  ph.rhoe_ref = ph.E_ref;
  const EntropyRefF c = entropy_ref_f(ph);
  for (int trial = 0; trial < 30000; ++trial) {
    const double amp = (trial % 3 == 0) ? 1e-3 : ((trial % 3 == 1) ? 3e-2 : 0.3);
    double u[D + 2];
    const double rho = 1.0 + amp * U(rng), p = ph.p_ref * (1.0 + amp * U(rng));
    double ke = 0;
    u[0] = rho;
    for (int m = 0; m < D; ++m) { const double v = U(rng); u[m + 1] = rho * v; ke += 0.5 * rho * v * v; }
    u[D + 1] = p / gm1 + ke;
    float du[D + 2], dw[D + 2];
    double ud[D + 2], w[D + 2];
    for (int e = 0; e < D + 2; ++e) {
      du[e] = (float)(u[e] - uref[e]);
      ud[e] = uref[e] + (double)du[e];
    }
    cons_to_entropy_fast<D>(g, gm1, igm1, ud, w);
    cons_to_entropy_pert<D>(c, du, dw);
    double scale = 0, err = 0;
    for (int e = 0; e < D + 2; ++e) scale = std::fmax(scale, std::fabs(w[e] - ph.w_ref[e]));
    for (int e = 0; e < D + 2; ++e) err = std::fmax(err, std::fabs((double)dw[e] - (w[e] - ph.w_ref[e])));
    worst[11] = std::fmax(worst[11], err / scale);
    // inverse map from the FP32 rounding of the exact perturbation
    float dwf[D + 2], dub[D + 2];
    double wd[D + 2], ub[D + 2];
    for (int e = 0; e < D + 2; ++e) {
      dwf[e] = (float)(w[e] - ph.w_ref[e]);
      wd[e] = ph.w_ref[e] + (double)dwf[e];
    }
    // FP32 JVPs of both maps at the absolute FP32 state against the FP64 ones
    {
      double v[D + 2], jd[D + 2], jd2[D + 2], rhoe = ud[D + 1];
      float uf[D + 2], wf[D + 2], vf[D + 2], jf[D + 2], jf2[D + 2];
      for (int m = 0; m < D; ++m) rhoe -= 0.5 * ud[m + 1] * ud[m + 1] / ud[0];
      for (int e = 0; e < D + 2; ++e) {
        v[e] = U(rng);
        vf[e] = (float)v[e];
        v[e] = (double)vf[e];
        uf[e] = (float)ud[e];
        wf[e] = (float)w[e];
      }
      double udf[D + 2], wdf[D + 2];
      for (int e = 0; e < D + 2; ++e) { udf[e] = (double)uf[e]; wdf[e] = (double)wf[e]; }
      cons_to_entropy_jvp<D>(g, gm1, igm1, udf, v, jd);
      cons_to_entropy_jvp_f<D>((float)g, (float)gm1, (float)igm1, uf, vf, jf);
      entropy_to_cons_jvp<D>(g, gm1, igm1, lg, wdf, v, jd2);
      entropy_to_cons_jvp_rhoe_f<D>((float)gm1, (float)igm1, (float)g, wf, (float)rhoe, vf, jf2);
      double s1 = 0, e1 = 0, s2 = 0, e2 = 0;
      for (int e = 0; e < D + 2; ++e) {
        s1 = std::fmax(s1, std::fabs(jd[e]));
        e1 = std::fmax(e1, std::fabs((double)jf[e] - jd[e]));
        s2 = std::fmax(s2, std::fabs(jd2[e]));
        e2 = std::fmax(e2, std::fabs((double)jf2[e] - jd2[e]));
      }
      worst[13] = std::fmax(worst[13], e1 / s1);
      worst[14] = std::fmax(worst[14], e2 / s2);
    }
    entropy_to_cons_fast<D>(g, gm1, igm1, lg, wd, ub);
    entropy_to_cons_pert<D>(c, dwf, dub);
    scale = 0;
    err = 0;
    for (int e = 0; e < D + 2; ++e) scale = std::fmax(scale, std::fabs(ub[e] - uref[e]));
    for (int e = 0; e < D + 2; ++e) err = std::fmax(err, std::fabs((double)dub[e] - (ub[e] - uref[e])));
    worst[12] = std::fmax(worst[12], err / scale);
  }
}

// the table-driven logarithm / exponential against the C library's in
// extended precision: ulps of the double result, over the ranges the
// entropy maps see and far beyond; out-of-range arguments take the library
// functions (NaN for negative logs, which the non-physical flag relies on)
void check_logexp(std::mt19937_64 &rng, double *worst) {
  static double tab[3 * sse::kLogTab + 2 * sse::kExpTab];
  sse::sse_build_math_tables(tab);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  auto ulps = [](double got, long double want) {
    const double w = (double)want;
    const double ulp = std::nextafter(std::fabs(w), INFINITY) - std::fabs(w);
    return (double)(std::fabs((long double)got - want) / ulp);
  };
  for (int i = 0; i < 2000000; ++i) {
    const double x = std::exp(40.0 * U(rng));                 // 4e-18 .. 2e17
    const long double lw = std::log((long double)x);
    // log: ulps of the result, or of 1 where the result is below 1 in
    // magnitude (an absolute-accuracy form: e ln2 + log F is not formed
    // relative to a result near zero)
    const double g = sse::sse_log(x, tab);
    const double ul = std::fabs((double)lw) >= 1.0 ? ulps(g, lw) : (double)(std::fabs((long double)g - lw) / 0x1p-52);
    worst[16] = std::fmax(worst[16], ul);
    const double y = 700.0 * U(rng);
    worst[17] = std::fmax(worst[17], ulps(sse::sse_exp(y, tab), std::exp((long double)y)));
  }
  // arguments outside the table range go to the library functions
  if (!std::isnan(sse::sse_log(-1.0, tab)) || sse::sse_log(0.0, tab) != -INFINITY ||
      sse::sse_exp(800.0, tab) != INFINITY || sse::sse_exp(-800.0, tab) != 0.0 ||
      !std::isnan(sse::sse_exp(NAN, tab)) || sse::sse_log(5e-320, tab) != std::log(5e-320))
    worst[18] += 1.0;
}

int main() {
  std::mt19937_64 rng(20261203);
  double worst[19] = {0};
  check_logexp(rng, worst);
  check<2>(rng, worst);
  check<3>(rng, worst);
  check_mixed<2>(rng, worst);
  check_mixed<3>(rng, worst);
  check_adjoint<2>(rng, worst);
  check_adjoint<3>(rng, worst);
  check_mixed_adjoint<2>(rng, worst);
  check_mixed_adjoint<3>(rng, worst);
  check_entropy_pert<2>(rng, worst);
  check_entropy_pert<3>(rng, worst);
  std::printf("{\"logmean\": %.3e, \"inv_logmean\": %.3e, \"ec_flux_dot\": %.3e, "
              "\"cons_to_entropy\": %.3e, \"entropy_to_cons\": %.3e, \"mixed_reduced_flux\": %.3e, "
              "\"flux_vjp_vs_fd\": %.3e, \"entropy_jvp_vs_fd\": %.3e, \"entropy_jacobian_symmetry\": %.3e, "
              "\"mixed_flux_vjp\": %.3e, \"ec_flux_half_mismatches\": %.0f, "
              "\"cons_to_entropy_pert\": %.3e, \"entropy_to_cons_pert\": %.3e, "
              "\"cons_to_entropy_jvp_f\": %.3e, \"entropy_to_cons_jvp_f\": %.3e, "
              "\"ec_flux_half_energy\": %.3e, \"table_log_ulps\": %.3f, \"table_exp_ulps\": %.3f, "
              "\"table_logexp_special_mismatches\": %.0f}\n",
              worst[0], worst[1], worst[2], worst[3], worst[4], worst[5], worst[6], worst[7], worst[8],
              worst[9], worst[10], worst[11], worst[12], worst[13], worst[14], worst[15], worst[16], worst[17],
              worst[18]);
  return 0;
}
