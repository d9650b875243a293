/* Stand-in for OP2's op_lib_cpp.h so that the reference's translated driver
 * (src/airfoil_op.cpp:6) compiles unchanged against op2_gb300.
 *
 * airfoil_op.cpp declares its op_par_loop_<kernel> functions itself
 * (src/airfoil_op.cpp:17-94) with C++ linkage unless OPENACC is defined; the
 * library exports them with C linkage, so this header turns that switch on. */
#ifndef OP_LIB_CPP_H
#define OP_LIB_CPP_H
#ifndef OPENACC
#define OPENACC 1
#endif
#include "op2_gb300.h"
#endif
