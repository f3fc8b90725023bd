// Oracle-build stand-in: vectors are not used beyond the matrix header.
#include "matrix.hpp"
