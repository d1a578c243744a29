// Definitions for the helpers the reference's Util.h declares (its Util.cpp
// does not compile with a current g++).  Written for this recipe.
#include <cstdio>
#include <string>
#include <sys/time.h>
#include <algorithm>
#include <cctype>
#include <cassert>
#include <cmath>
typedef long int int64;
void destroy_arr_valid(void** ptr) { if (*ptr) { delete[] (char*)*ptr; *ptr = 0; } }
size_t GetFilenameSize(std::string name) {
  FILE* f = fopen(name.c_str(), "r"); if (!f) return 0;
  fseek(f, 0, SEEK_END); size_t n = (size_t)ftell(f); fclose(f); return n;
}
bool fexists(const char* fn) { FILE* f = fopen(fn, "r"); if (f) fclose(f); return f != nullptr; }
std::string& ltrim(std::string& s) {
  s.erase(s.begin(), std::find_if(s.begin(), s.end(), [](unsigned char c) { return !std::isspace(c); }));
  return s;
}
std::string& rtrim(std::string& s) {
  s.erase(std::find_if(s.rbegin(), s.rend(), [](unsigned char c) { return !std::isspace(c); }).base(), s.end());
  return s;
}
std::string& trim(std::string& s) { return ltrim(rtrim(s)); }
void ReadFortranRecord(FILE* io, void* data) {
  unsigned int n = 0;
  if (fread(&n, 4, 1, io) != 1) return;
  if (fread(data, n, 1, io) != 1) return;
  if (fread(&n, 4, 1, io) != 1) return;
}
void assertdouble(double& a, double& b, double tol) { assert(std::fabs(a - b) < tol); }
int64 GetTimeMs64() { struct timeval tv; gettimeofday(&tv, 0); return tv.tv_sec * 1000 + tv.tv_usec / 1000; }
int G_VERBOSE = 0;
