// gbf_defines.cpp — the reference's parameter file (defines.ini) on any OS.
//
// read_defines (main.cpp:601-684) opens the hard-coded Windows path of
// defines.h:5, skips lines that start with '#', splits the others at the
// first '=' and reads the value up to the first space with atof/atoi; a line
// without '=' makes it read past the string. This parser takes a path, the
// same keys and the same value rule (the token after '=' up to white space,
// so CRLF line ends and trailing comments are harmless), and skips blank
// lines and lines without '='. The grid size NX, NY, NZ is required.
//
// The file also lists the physical constants (K[i], LAMBDA[i], S_WR[i], M[i],
// P_D[i], MU1, MU2, RO_W, RO_N, S2_GR, P_ATM, G_CONST), which read_defines
// ignores in favour of the equal compile-time values of defines.h:6-26; they
// are read here too, so that editing the file changes the model. Other keys
// (OMEGA, EPSILON, ...) are ignored.
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "gbf_internal.h"

namespace {
std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && isspace((unsigned char)s[a])) a++;
  while (b > a && isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}
}  // namespace

extern "C" int gbf_read_defines(const char* path, gbf_model* m, gbf_run_defines* run) {
  if (!path || !m) return gbf_fail(GBF_ERR_ARG, "gbf_read_defines");
  FILE* f = fopen(path, "r");
  if (!f) return gbf_fail(GBF_ERR_ARG, "gbf_read_defines: cannot open file");
  gbf_model md;
  gbf_model_reference(&md, 0, 0, 0, 0.0);
  gbf_run_defines rd = {0.0, 0.0, 0.0, 0.0, 0, 0};
  char line[1024];
  while (fgets(line, sizeof(line), f)) {
    std::string s(line);
    if (!s.empty() && s[0] == '#') continue;
    const size_t eq = s.find('=');
    if (eq == std::string::npos) continue;
    const std::string key = trim(s.substr(0, eq));
    std::string val = trim(s.substr(eq + 1));
    const size_t sp = val.find_first_of(" \t\r\n#");
    if (sp != std::string::npos) val = val.substr(0, sp);
    const double v = atof(val.c_str());
    const int iv = atoi(val.c_str());
    if (key == "H1") md.h1 = v;
    else if (key == "H2") md.h2 = v;
    else if (key == "H3") md.h3 = v;
    else if (key == "DT") md.dt = v;
    else if (key == "BETA1") md.beta1 = v;
    else if (key == "BETA2") md.beta2 = v;
    else if (key == "SOURCE") md.source = iv;
    else if (key == "NX") md.nx = iv;
    else if (key == "NY") md.ny = iv;
    else if (key == "NZ") md.nz = iv;
    else if (key == "TAU") rd.tau = v;
    else if (key == "L_W") rd.l_w = v;
    else if (key == "L_N") rd.l_n = v;
    else if (key == "C") rd.c = v;
    else if (key == "SAVE_PLOTS") rd.save_plots = iv;
    else if (key == "PRINT_SCREEN") rd.print_screen = iv;
    else if (key == "MU1") md.mu1 = v;
    else if (key == "MU2") md.mu2 = v;
    else if (key == "RO_W") md.ro01 = v;
    else if (key == "RO_N") md.ro02 = v;
    else if (key == "S2_GR") md.S2_gr = v;
    else if (key == "P_ATM") md.P_atm = v;
    else if (key == "G_CONST") md.g = v;
    else {
      // per-media table entries NAME[i], i in {0, 1}
      static const char* names[] = {"K", "LAMBDA", "S_WR", "M", "P_D"};
      double* dst[] = {md.K, md.lambda, md.S_wr, md.m, md.P_d};
      for (int q = 0; q < 5; q++) {
        const std::string n = names[q];
        if (key.size() == n.size() + 3 && key.compare(0, n.size(), n) == 0 && key[n.size()] == '[' &&
            (key[n.size() + 1] == '0' || key[n.size() + 1] == '1') && key[n.size() + 2] == ']')
          dst[q][key[n.size() + 1] - '0'] = v;
      }
    }
  }
  fclose(f);
  if (md.nx < 1 || md.ny < 1 || md.nz < 1) return gbf_fail(GBF_ERR_ARG, "gbf_read_defines: NX, NY, NZ missing");
  *m = md;
  if (run) *run = rd;
  return GBF_OK;
}
