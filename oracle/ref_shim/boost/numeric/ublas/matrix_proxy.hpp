// Oracle-build stand-in: range views live in matrix.hpp.
#include "matrix.hpp"
