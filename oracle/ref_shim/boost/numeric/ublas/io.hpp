// Oracle-build stand-in: stream output lives in matrix.hpp.
#include "matrix.hpp"
