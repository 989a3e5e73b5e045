// Minimal stand-in for CLI11's <CLI/CLI.hpp>, written for this project.
//
// TEST INFRASTRUCTURE ONLY: it lets the reference's apps/cpu_demo/main.cpp
// compile unmodified (as a library, its main renamed) so that its checkTree
// can be called on octrees; command-line parsing is never run. It provides
// only what that file names: CLI::App, add_option(...)->check(...),
// CLI::PositiveNumber, CLI::Range and CLI11_PARSE.
#pragma once

namespace CLI {

struct Validator {};
inline const Validator PositiveNumber{};
inline Validator Range(int, int) { return Validator{}; }

struct Option {
  Option* check(const Validator&) { return this; }
};

struct App {
  explicit App(const char*) {}
  template <class T>
  Option* add_option(const char*, T&, const char*) {
    return &option;
  }
  Option option;
};

}  // namespace CLI

#define CLI11_PARSE(app, argc, argv) \
  (void)(app);                       \
  (void)(argc);                      \
  (void)(argv);
