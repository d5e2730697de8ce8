// The glisser command: the reference's targets/main.cpp:29-60 entry point
// (usage "glisser [options] [<config>]", config.in by default) over the C ABI.
// Everything main() does after reading the configuration -- the output folder
// layout, stdout tee, state.in, encounter/time/timing logs, tracks, dumps,
// planetary history, the end state -- is glisser_run.  The reference asks on
// stdin before writing into a non-empty output folder; this command refuses
// unless --force is given (it never reads stdin).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

#include "glisser.h"

namespace {

const char USAGE[] =
    "glisser\n"
    "Usage:\n"
    "    glisser [options] [<config>]\n"
    "\n"
    "Options:\n"
    "    -h, --help         Show this screen.\n"
    "    --force            Write into a non-empty output folder.\n"
    "    --quiet            Do not echo the run log to stdout (it is still written to <Output-Folder>/stdout).\n";

std::string last_error(const glisser_t* h)
{
    char buf[2048] = { 0 };
    if (h) glisser_last_error(h, buf, sizeof buf);
    else glisser_last_error_global(buf, sizeof buf);
    return buf;
}

}  // namespace

int main(int argc, char** argv)
{
    std::string configin = "config.in";
    bool force = false, quiet = false, have_config = false;
    for (int i = 1; i < argc; i++) {
        const char* a = argv[i];
        if (!std::strcmp(a, "-h") || !std::strcmp(a, "--help")) {
            std::cout << USAGE;
            return 0;
        } else if (!std::strcmp(a, "--force")) {
            force = true;
        } else if (!std::strcmp(a, "--quiet")) {
            quiet = true;
        } else if (a[0] == '-' || have_config) {
            std::cerr << USAGE;
            return 1;
        } else {
            configin = a;
            have_config = true;
        }
    }
    std::cout << "Reading from configuration file " << configin << std::endl;
    std::ifstream f(configin);
    if (!f) {
        std::cerr << "Could not read configuration." << std::endl << "cannot open " << configin << std::endl;
        return -1;
    }
    std::stringstream text;
    text << f.rdbuf();
    glisser_t* h = nullptr;
    if (glisser_create(text.str().c_str(), &h) != GLISSER_OK) {
        std::cerr << "Could not read configuration." << std::endl << last_error(nullptr) << std::endl;
        return -1;
    }
    int rc = glisser_run(h, (quiet ? 1 : 0) | (force ? 2 : 0));
    if (rc != GLISSER_OK) std::cerr << last_error(h) << std::endl;
    glisser_destroy(h);
    return rc == GLISSER_OK ? 0 : -1;
}
