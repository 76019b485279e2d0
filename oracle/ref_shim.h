/*
 * Force-included header used only when compiling the reference DEM sources
 * (test infrastructure; never part of the GPU engine).
 *
 * GCC >= 4.7 applies two-phase lookup strictly: templates inside namespace
 * `aries` that write `scalar * Vector3d` cannot see the global
 * `operator*(const T, const aries::Vector3d<T>)` that aries/utility/Vector3d.h
 * declares only after those templates (Vector3d.h:314), and ADL does not find a
 * global-namespace operator for an `aries` class.  Declaring the template up
 * front and re-exporting it into `aries` makes the unmodified sources compile.
 */
#ifndef VEDO_ORACLE_REF_SHIM_H
#define VEDO_ORACLE_REF_SHIM_H
#ifdef __cplusplus
namespace aries { template <typename T> class Vector3d; }
template <typename T> aries::Vector3d<T> operator * (const T s, const aries::Vector3d<T> v);
namespace aries { using ::operator*; }
#endif
#endif
