// The reference's thermodynamics files (host code, no device).
//
// CNRGthermo::SaveNValue (NRGthermoClass.cpp:109-150) appends one line per
// temperature: T, the value, the chain value (0 in a chain file), and the
// value minus the chain value, each written by an ofstream with precision 20
// in scientific format, separated by single spaces.
#include <cstdio>

#include "../../include/twochnrg_gb300.h"

extern "C" {

nrg_status nrg_write_thermo(const char* path, int nvalues, const double* temp, const double* value,
                            const double* chain) {
  if (!path || nvalues < 0 || (nvalues > 0 && (!temp || !value))) return NRG_ERR_ARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return NRG_ERR_ARG;
  bool ok = true;
  for (int k = 0; k < nvalues && ok; ++k) {
    const double ch = chain ? chain[k] : 0.0;
    ok = std::fprintf(f, "%.20e %.20e %.20e %.20e\n", temp[k], value[k], ch, value[k] - ch) > 0;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? NRG_OK : NRG_ERR_ARG;
}

}  // extern "C"
