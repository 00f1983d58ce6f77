/* HEALPix C++ compatibility shim (TEST INFRASTRUCTURE ONLY).
 * Lets the reference's own Convolver/PolBeam/Sky sources compile against
 * the oracle's HEALPix restatement, because the Healpix C++ library they
 * include is not available.  Only the members the reference uses exist. */
#ifndef PISCO_SHIM_POINTING_H
#define PISCO_SHIM_POINTING_H
struct pointing {
    double theta, phi;
    pointing() : theta(0.0), phi(0.0) {}
    pointing(double t, double p) : theta(t), phi(p) {}
};
#endif
