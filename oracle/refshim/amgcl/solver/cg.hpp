// Stand-in header (TEST INFRASTRUCTURE for oracle/_ref): every amgcl name used by the reference is declared in make_solver.hpp.
#pragma once
#include "../make_solver.hpp"
