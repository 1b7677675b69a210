// Reconstruction options: the reference's command-line / config-file option
// names, defaults and storage semantics (setupProgramOptions and setParams,
// src/cudaSirecon/cudaSirecon.cpp:913-1070, over SetDefaultParams 16-72),
// without Boost.
#pragma once
#include <set>
#include <string>
#include <vector>

#include "cudasirecon.h"

namespace simrecon {

struct Options {
  ReconParams p;
  ImageParams ip;
  std::string config_file;
  bool help = false;
  bool version = false;
  // extensions (no reference counterpart)
  bool reference_flag_bytes = true;  // model the reference's int-sized reads of bool flags
  std::set<std::string> given;       // options explicitly set (CLI or config)
};

void set_defaults(Options* o);
// one option by its long name; `value` is the text after '=' (or the next
// token); `has_value` false for a bare switch.
bool apply_option(Options* o, const std::string& key, const std::string& value, bool has_value, std::string* err);
// key=value lines ('#' comments); options already given on the command line win
bool apply_config_text(Options* o, const std::string& text, std::string* err);
bool apply_config_file(Options* o, const std::string& path, bool must_exist, std::string* err);
// the cudasirecon command line: input output otf [--opt[=v] | --opt v | -c cfg]...
bool parse_command_line(Options* o, int argc, char** argv, std::string* err);
std::string usage_text();

// the kz=0 exclusion the reference's kernels actually apply: bNoKz0 is read
// as a 4-byte int spanning its padding byte and the low half of wiener
bool effective_nokz0(const Options& o);

}  // namespace simrecon
