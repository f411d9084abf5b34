/*
 * Atomic-unit conversion constants for the CPU oracle (test infrastructure).
 *
 * libdft takes these from libgrid's <grid/au.h>, which is not available; the
 * values below are restated from CODATA 2018.  Hartree atomic units:
 * hbar = m_e = e = 1, length in bohr, energy in hartree.
 *
 * Call sites in libdft: src/ot.c:1240-1257 (parameter conversion),
 * src/helium-ot-bulk.c:356-360 (dispersion units).
 */
#ifndef ORACLE_GRID_AU_H
#define ORACLE_GRID_AU_H

#define GRID_AUTOANG   0.529177210903        /* bohr -> Angstrom */
#define GRID_AUTOM     0.529177210903E-10    /* bohr -> m */
#define GRID_AUTOK     3.1577502480407E5     /* hartree -> K */
#define GRID_AUTOFS    0.024188843265857     /* a.u. time -> fs */
#define GRID_AUTOS     2.4188843265857E-17   /* a.u. time -> s */
#define GRID_AUTOAMU   (1.0 / 1822.888486209) /* electron mass -> amu (m_e / u) */
#define GRID_AUTOMPS   2.18769126364E6       /* a.u. velocity -> m/s */
#define GRID_AUTOPA    2.9421015697E13       /* a.u. pressure -> Pa */
#define GRID_AUTOBAR   2.9421015697E8        /* a.u. pressure -> bar */
#define GRID_AUKB      (1.0 / GRID_AUTOK)    /* Boltzmann constant, hartree / K */
#define GRID_HZTOCM1   3.33564095198152E-11  /* Hz -> cm^-1 (1/c in cm/s) */
#define GRID_AUTOCM1   2.1947463136320E5     /* hartree -> cm^-1 */
#define GRID_AUTOEV    27.211386245988       /* hartree -> eV */

#endif
