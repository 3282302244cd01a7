/*
 * Test infrastructure (oracle build only): the part of the gflags API that
 * xpcs-eigen's main.cpp uses (DEFINE_bool / DEFINE_int32 / DEFINE_string and
 * ParseCommandLineFlags).  Accepts "--name", "--name=value" and "--noname"
 * for booleans; parsed flags are removed from argv.
 */
#ifndef XPCS_ORACLE_FAKE_GFLAGS_H
#define XPCS_ORACLE_FAKE_GFLAGS_H

#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace gflags {

struct FlagSlot {
  const char *name;
  int kind;  // 0 bool, 1 int32, 2 string
  void *ptr;
};

inline std::vector<FlagSlot> &flag_registry() {
  static std::vector<FlagSlot> slots;
  return slots;
}

struct FlagRegistrar {
  FlagRegistrar(const char *name, int kind, void *ptr) {
    flag_registry().push_back(FlagSlot{name, kind, ptr});
  }
};

inline bool assign_flag(const std::string &name, const std::string &value, bool has_value) {
  for (FlagSlot &s : flag_registry()) {
    if (name == s.name) {
      if (s.kind == 0)
        *(bool *)s.ptr = !has_value || value == "true" || value == "1";
      else if (s.kind == 1)
        *(int *)s.ptr = atoi(value.c_str());
      else
        *(std::string *)s.ptr = value;
      return true;
    }
    if (s.kind == 0 && name == std::string("no") + s.name) {
      *(bool *)s.ptr = false;
      return true;
    }
  }
  return false;
}

inline void ParseCommandLineFlags(int *argc, char ***argv, bool) {
  std::vector<char *> rest;
  rest.push_back((*argv)[0]);
  for (int i = 1; i < *argc; i++) {
    char *a = (*argv)[i];
    if (strncmp(a, "--", 2) != 0) {
      rest.push_back(a);
      continue;
    }
    std::string body(a + 2), value;
    bool has_value = false;
    size_t eq = body.find('=');
    if (eq != std::string::npos) {
      value = body.substr(eq + 1);
      body = body.substr(0, eq);
      has_value = true;
    }
    if (!assign_flag(body, value, has_value)) rest.push_back(a);
  }
  for (size_t i = 0; i < rest.size(); i++) (*argv)[i] = rest[i];
  *argc = (int)rest.size();
}

}  // namespace gflags

#define DEFINE_bool(name, dflt, help) \
  bool FLAGS_##name = dflt;           \
  static gflags::FlagRegistrar flag_reg_##name(#name, 0, &FLAGS_##name)
#define DEFINE_int32(name, dflt, help) \
  int FLAGS_##name = dflt;             \
  static gflags::FlagRegistrar flag_reg_##name(#name, 1, &FLAGS_##name)
#define DEFINE_string(name, dflt, help) \
  std::string FLAGS_##name = dflt;      \
  static gflags::FlagRegistrar flag_reg_##name(#name, 2, &FLAGS_##name)

#endif
