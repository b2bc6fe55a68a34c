// Physical and numerical constants of the opacity path (MeV, nm, s units).
//
// Values and the double-precision expressions that derive them follow
// bns_nurates include/constants.hpp:30-244, so that the folded constants are
// bit-identical to the reference's; a GPU test compares them.  Usable from
// host C++ and CUDA device code.
#pragma once

namespace bnsn {
namespace k {

constexpr double MeV   = 1.6021766341182763e+8; // MeV in nm^2 g s^-2
constexpr double Me    = 0.51099895069;         // electron mass [MeV]
constexpr double Mn    = 939.56542194;          // neutron mass [MeV]
constexpr double Mp    = 938.27208943;          // proton mass [MeV]
constexpr double Q     = 1.29333251;            // Mn - Mp [MeV]
constexpr double Mu    = 1.66053906892e-24;     // atomic mass unit [g]
constexpr double Mb    = 1.6737747126723517e-24; // mean baryon mass [g]
constexpr double Pi    = 3.14159265358979323846264338328;
constexpr double H     = 4.135667696e-21;       // [MeV s]
constexpr double Hbar  = 0.5 * H / Pi;
constexpr double Clight = 2.99792458e+17;       // [nm s^-1]
constexpr double Gf0   = 1.1663787e-11;         // [MeV^-2]
constexpr double Gf    = Gf0 * ((Hbar * Clight) * (Hbar * Clight) * (Hbar * Clight));
constexpr double SatN  = 0.15e+18;              // [nm^-3]

constexpr double Ga = 1.23, Gv = 1., Gs = 0., SinThW2 = 0.2325;
constexpr double Hnv = -0.5;
constexpr double Hna = -0.5 * Ga;
constexpr double Hpv = 0.5 - 2. * SinThW2;
constexpr double Hpa = 0.5 * Ga;

// Bruenn (C13,C15,C19,C20) prefactor
constexpr double BetaConst =
    ((Clight * Clight * Clight) * ((Gf0 * Hbar) * (Gf0 * Hbar))) *
    ((Gv * Gv) + 3. * (Ga * Ga)) / Pi;

// iso-energetic scattering
constexpr double IsoEf    = 4.785390000313652 * (Hbar * Hbar) / Mb * MeV;
constexpr double IsoConst = 2. * Pi * (Gf * Gf) / Hbar /
                            ((H * Clight) * (H * Clight) * (H * Clight));
constexpr double IsoH0p = (Hpv * Hpv) + 3. * (Hpa * Hpa);
constexpr double IsoH1p = (Hpv * Hpv) - (Hpa * Hpa);
constexpr double IsoH0n = (Hnv * Hnv) + 3. * (Hna * Hna);
constexpr double IsoH1n = (Hnv * Hnv) - (Hna * Hna);
constexpr double IsoC0p = IsoConst * IsoH0p;
constexpr double IsoC1p = IsoConst * IsoH1p;
constexpr double IsoC0n = IsoConst * IsoH0n;
constexpr double IsoC1n = IsoConst * IsoH1n;

// nucleon-nucleon bremsstrahlung
constexpr double BremXmin = 1.0e-10, BremYmin = 1.0e-10, BremEtamin = 1.0e-10;
constexpr double BremAux1  = 0.25 * (H * H) * MeV / (Pi * Pi);
constexpr double BremCa    = -0.63;
constexpr double BremConst = (BremCa * BremCa) * (Gf * Gf) / Hbar;
constexpr double BremC4BRT06 = 0.1409912109375;

// e+e- pair process (Pons et al. 1998, Table 1)
constexpr double PairPhi = 1.55e-12 / Pi;
constexpr double PairA1e = 1. + 2. * SinThW2;
constexpr double PairA2e = 2. * SinThW2;
constexpr double PairA1x = -1. + 2. * SinThW2;
constexpr double PairA2x = 2. * SinThW2;

// inelastic scattering on e+- (Mezzacappa & Bruenn 1993)
constexpr double NepsConst =
    2. * (Gf0 * Gf0) * Clight * ((Hbar * Clight) * (Hbar * Clight)) / (3. * Pi);
constexpr double NepsBPlus  = (2. * SinThW2 + 1.) * (2. * SinThW2 + 1.);
constexpr double NepsBMinus = (2. * SinThW2 - 1.) * (2. * SinThW2 - 1.);
constexpr double NepsBZero  = 4. * (SinThW2 * SinThW2);

// miscellaneous
constexpr double ExpUpp = 700., ExpLow = -700.;
constexpr double HC6FourPi2 =
    (H * Clight) * (H * Clight) * (H * Clight) * (H * Clight) * (H * Clight) *
    (H * Clight) / (16. * (Pi * Pi));
constexpr double WmEScale  = MeV / (Mb * (Clight * Clight));
constexpr double FourPiHc3 = (4. * Pi) / ((H * Clight) * (H * Clight) * (H * Clight));
constexpr double FourPiHc3Sqr = FourPiHc3 * FourPiHc3;
constexpr double MnGrams   = Mn * MeV / (Clight * Clight);
constexpr double MpGrams   = Mp * MeV / (Clight * Clight);
constexpr double MAvgGrams = MeV / (Clight * Clight) * 938.918532994116257276238085018813;
constexpr double SqrtPi    = 1.77245385090551602729816748334106;
constexpr double PiSq      = 9.86960440108935861883449099987572;
constexpr double FourPiSq  = 39.4784176043574344753379639995029;
constexpr double Pi18      = 1.15383506784998943054096521314981; // pi^(1/8)
constexpr double PiHalf52  = 3.09242868139914350627854469835251; // (pi/2)^2.5
constexpr double FdiLit    = 7.38905609893065023;                // e^2

// thresholds of the grey driver (m1_opacities.hpp:19-20)
constexpr double ThresholdN = 1e-21, ThresholdJ = 1e-25;
// energy-scale multiple of the 2-D integrals (m1_opacities.hpp:1085)
constexpr double TempMultiple = 0.5 * 4.364;
constexpr double CF = 0.6; // thin-distribution power (distribution.hpp:18)

} // namespace k
} // namespace bnsn
