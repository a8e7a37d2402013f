/* Minimal stand-in for GadgetReader's gadgetreader.hpp, used only to compile
 * the reference's fieldize.cpp into the test oracle (oracle/_ref).  gen-pk.h
 * needs the GSnap class name (in a prototype), the particle-type constants and
 * N_TYPE; the GadgetReader submodule itself is not vendored in the reference. */
#ifndef ORACLE_SHIM_GADGETREADER_HPP
#define ORACLE_SHIM_GADGETREADER_HPP
#include <cstdint>
#include <string>
#include <vector>
#define N_TYPE 6
#define BARYON_TYPE 0
#define DM_TYPE 1
#define DISK_TYPE 2
#define NEUTRINO_TYPE 2
#define BULGE_TYPE 3
#define STARS_TYPE 4
#define BNDRY_TYPE 5
namespace GadgetReader { class GSnap; }
#endif
