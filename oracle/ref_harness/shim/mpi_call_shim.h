/*
 * Force-included ahead of every reference translation unit in the oracle
 * build. It pre-defines the include guard of the reference's mpi_call.h,
 * whose template body does not compile with g++ 13 (shadowed template
 * parameter, mpi_call.h:143; unknown Triangle member, mpi_call.h:193), and
 * supplies an empty MPI_CALL<T> so that Geometry's unused `mpi_caller` member
 * (ComplexGeometry.h:36) still has a type.
 */
#pragma once
#define _MPI_CALL_H
template <class T>
class MPI_CALL {};
