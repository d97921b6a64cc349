/*
 * The lsrelax- and nmrelax-compatible drivers: batch files (parse_batch_file,
 * large_strain_relax.cu:263-383, network_mesh_relax.cu:413-500), file lists
 * (file_lists.cpp:11-138), the per-network runs with the reference's output
 * files (do_relaxation_run, large_strain_relax.cu:792-1010 and
 * network_mesh_relax.cu:1095-1390), relaxation_batch and the command lines
 * (large_strain_relax.cu:1016-1126, network_mesh_relax.cu:1393-1503).
 *
 * Output formats are the reference's, byte for byte:
 *   _log.txt    "Convergence [not ]reached: Steps: %d, RMS Force: %12.8le"
 *               per relaxation, then "Elapsed time: %f seconds" (clock())
 *   _edata.txt  compression "%12.0lf\t%12.10lf\t%12.8le\t%12.8le\t%12.8le"
 *               shear       "%12.10lf\t%12.10lf\t%12.10le\t%12.10le\t%12.10le"
 *   _NNN.pos    "%2.10le\t%2.10le" per node after each shear step
 * nmrelax's _edata.txt has a gel column and a total:
 *               compression "%12.0lf\t%12.10lf" then four "%12.8le"
 *               shear       "%12.8lf\t%12.8lf" then four "%12.8le"
 * Deliberate differences: a network file that fails to parse is skipped
 * with an error instead of being relaxed half-read; an increment of 0 runs
 * one step instead of looping forever; -a selects absolute displacements
 * instead of falling through into -b with no argument.
 */
#include <algorithm>
#include <cctype>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <regex>
#include <sstream>
#include <string>
#include <vector>

#include "nr_internal.h"

using nr::fail;

namespace {

/* read_line, large_strain_relax.cu:263-283: next line that is neither empty
 * nor a '#' comment. */
bool read_line(std::ifstream &input, std::string &line) {
    if (input.eof()) {
        fprintf(stderr, "Not enough information was provided in the batch file.\n");
        return false;
    }
    while (!input.eof()) {
        std::getline(input, line);
        if (line.empty() || line[0] == '#') continue;
        break;
    }
    return !(line.empty() || line[0] == '#');
}

/* split_line (large_strain_relax.cu:229): tokens separated by spaces and
 * tabs, of the line up to its first NUL (the reference strtok's a strcpy'd
 * copy). */
std::vector<std::string> split_ws(const std::string &line) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : line) {
        if (c == '\0') break;
        if (c == ' ' || c == '\t') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

int get_dec_digits(int value) {
    int digits = 0;
    do {
        digits++;
        value /= 10;
    } while (value > 0);
    return digits;
}

std::string report_name(const std::string &base, int num_digits, int count, const char *ext) {
    std::ostringstream oss;
    oss << base << "_";
    for (int i = 0; i < num_digits - get_dec_digits(count); ++i) oss << 0;
    oss << count << "." << ext;
    return oss.str();
}

struct FileLists {
    std::vector<std::string> dat, log, disp, edat;
};

bool file_lists(const std::string &input, const std::string &ext, const std::string &tag, FileLists &fl) {
    if (input.empty()) return false;
    std::vector<std::string> parts;
    std::string cur;
    for (char c : input) {
        if (c == '/') {
            if (!cur.empty()) parts.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    if (!cur.empty()) parts.push_back(cur);
    if (parts.empty()) return false;
    std::string base = parts.back(), dir;
    if (parts.size() > 1) {
        if (input[0] == '/') dir = "/";
        for (size_t i = 0; i + 1 < parts.size(); ++i) dir += parts[i] + "/";
    } else {
        dir = "./";
    }
    if (base == "*") base = "";
    std::regex expr("^(" + base + ".*)\\." + ext);
    const std::string suffix = tag.empty() ? std::string() : "_" + tag;
    std::error_code ec;
    if (std::filesystem::exists(dir, ec)) {
        for (const auto &entry : std::filesystem::directory_iterator(dir, ec)) {
            if (entry.is_directory()) continue;
            const std::string name = entry.path().filename().string();
            std::smatch m;
            if (std::regex_search(name, m, expr)) {
                fl.dat.push_back(dir + m[0].str());
                fl.log.push_back(dir + m[1].str() + suffix + "_log.txt");
                fl.disp.push_back(dir + m[1].str() + suffix);
                fl.edat.push_back(dir + m[1].str() + suffix + "_edata.txt");
            }
        }
    }
    std::sort(fl.dat.begin(), fl.dat.end());
    std::sort(fl.log.begin(), fl.log.end());
    std::sort(fl.disp.begin(), fl.disp.end());
    std::sort(fl.edat.begin(), fl.edat.end());
    return true;
}

}  // namespace

/* Both batch-file grammars: six non-comment lines; the second holds
 * "ks kb" (lsrelax) or "ks kb bmod smod dilation" (nmrelax, mesh != null). */
static int parse_batch(const char *path, nr_batch_spec *spec, nr_mesh_batch_spec *mesh) {
    memset(spec, 0, sizeof(*spec));
    std::ifstream input(path);
    if (!input.is_open()) {
        fprintf(stderr, "The file %s could not be read.\n", path);
        return fail(NR_ERR_IO, std::string("cannot open ") + path);
    }
    std::string line;
    if (!read_line(input, line)) return fail(NR_ERR_PARSE, "batch file: missing base name");
    std::vector<std::string> tok = split_ws(line);
    snprintf(spec->base, sizeof(spec->base), "%s", tok.empty() ? "" : tok[0].c_str());
    if (tok.size() > 1) snprintf(spec->tag, sizeof(spec->tag), "%s", tok[1].c_str());
    if (!read_line(input, line)) return fail(NR_ERR_PARSE, "batch file: missing stiffness line");
    if (mesh) {
        /* network_mesh_relax.cu:440-446: "ks kb bmod smod dilation", at least
         * three values (missing smod / dilation are 0 here; the reference
         * leaves them uninitialised) */
        if (sscanf(line.c_str(), "%lf %lf %lf %lf %lf", &spec->ks, &spec->kb, &mesh->bmod, &mesh->smod,
                   &mesh->dilation) < 3 ||
            spec->ks < 0 || spec->kb < 0 || mesh->bmod < 0 || mesh->smod < 0 || mesh->dilation < 0) {
            fprintf(stderr, "Error: invalid format for mechanical attributes.");
            return fail(NR_ERR_PARSE, "batch file: invalid mechanical attributes");
        }
    } else if (sscanf(line.c_str(), "%lf %lf", &spec->ks, &spec->kb) < 2 || spec->ks < 0 || spec->kb < 0) {
        fprintf(stderr, "Error: invalid format for mechanical attributes.");
        return fail(NR_ERR_PARSE, "batch file: invalid mechanical attributes");
    }
    if (!read_line(input, line)) return fail(NR_ERR_PARSE, "batch file: missing FIRE parameters");
    /* parse_doubles (large_strain_relax.cu:247): a token counts when sscanf
     * returns nonzero, so a token of only '\r' (sscanf gives EOF) repeats
     * the previous value; before any value it is 0 here (the reference's
     * variable is uninitialised). */
    std::vector<double> fp;
    double v = 0.0;
    for (const std::string &s : split_ws(line))
        if (sscanf(s.c_str(), "%lf", &v) != 0) fp.push_back(v);
    if (fp.size() < 5) {
        fprintf(stderr, "Too few FIRE parameters were supplied. 8 are needed.\n");
        return fail(NR_ERR_PARSE, "batch file: too few FIRE parameters");
    }
    for (int i = 0; i < 5; ++i) spec->fire_params[i] = fp[i];
    if (!read_line(input, line)) return fail(NR_ERR_PARSE, "batch file: missing nmin/mass/fcut/nmax");
    if (sscanf(line.c_str(), "%d %lf %lf %d", &spec->nmin, &spec->mass, &spec->fcut, &spec->nmax) < 4 ||
        spec->mass < 0 || spec->fcut < 0 || spec->nmax < 0) {
        fprintf(stderr, "On or more of nmin, mass, cutoff force and step limit were invalid.\n");
        return fail(NR_ERR_PARSE, "batch file: invalid nmin/mass/fcut/nmax");
    }
    for (int which = 0; which < 2; ++which) {
        double *r = which == 0 ? spec->compr : spec->shear;
        if (!read_line(input, line)) return fail(NR_ERR_PARSE, "batch file: missing strain range");
        if (sscanf(line.c_str(), "%lf %lf %lf", &r[0], &r[1], &r[2]) < 3 || r[0] < 0 || r[1] < 0 || r[2] < 0 ||
            r[1] < r[0]) {
            fprintf(stderr, which == 0 ? "Error: invalid specification of compression."
                                       : "Error: invalid specification of shear.");
            return fail(NR_ERR_PARSE, "batch file: invalid strain range");
        }
    }
    return NR_OK;
}

extern "C" {

int nr_parse_batch_file(const char *path, nr_batch_spec *spec) {
    if (!path || !spec) return fail(NR_ERR_INVALID, "nr_parse_batch_file: null argument");
    return parse_batch(path, spec, nullptr);
}

int nr_parse_mesh_batch_file(const char *path, nr_mesh_batch_spec *spec) {
    if (!path || !spec) return fail(NR_ERR_INVALID, "nr_parse_mesh_batch_file: null argument");
    memset(spec, 0, sizeof(*spec));
    return parse_batch(path, &spec->net, spec);
}

int nr_get_file_lists(const char *base, const char *ext, const char *tag, char *buf, size_t cap) {
    if (!base || !ext) return fail(NR_ERR_INVALID, "nr_get_file_lists: null argument");
    FileLists fl;
    if (!file_lists(base, ext, tag ? tag : "", fl)) return fail(NR_ERR_INVALID, "nr_get_file_lists: empty base");
    size_t pos = 0;
    for (size_t i = 0; i < fl.dat.size(); ++i) {
        for (const std::string *s : {&fl.dat[i], &fl.log[i], &fl.disp[i], &fl.edat[i]}) {
            if (buf) {
                if (pos + s->size() + 1 > cap) return fail(NR_ERR_CAPACITY, "nr_get_file_lists: buffer too small");
                memcpy(buf + pos, s->c_str(), s->size() + 1);
            }
            pos += s->size() + 1;
        }
    }
    return (int)fl.dat.size();
}

int nr_do_relaxation_run(const char *net_file, const char *log_name, const char *edata_name, const char *disp_base,
                         const nr_batch_spec *spec, int precision, int criterion) {
    if (!net_file || !log_name || !edata_name || !disp_base || !spec)
        return fail(NR_ERR_INVALID, "nr_do_relaxation_run: null argument");
    const clock_t ct0 = clock();
    nr_host_network *hn = nullptr;
    int rc = nr_read_network(net_file, &hn);
    if (rc != NR_OK) {
        fprintf(stderr, "%s: %s\n", net_file, nr_last_error());
        nr_host_network_free(hn);
        return rc;
    }
    if (spec->kb > 0) nr_get_triples(hn);
    const double miny = hn->miny, range = hn->maxy - hn->miny;
    const double smult = spec->absolute ? 1.0 : range;
    const double s_inc = spec->shear[2];
    const int num_digits =
        get_dec_digits(1 + (s_inc > 0 ? (int)((spec->shear[1] - spec->shear[0]) / s_inc) : 0));
    nr_network *net = nullptr;
    rc = nr_network_create(hn, spec->ks, spec->kb, nullptr, &net);
    const int n_points = hn->n_points;
    nr_host_network_free(hn);
    if (rc != NR_OK) return rc;
    nr_fire_params p;
    p.alpha0 = spec->fire_params[0];
    p.falpha = spec->fire_params[1];
    p.dt_max = spec->fire_params[2];
    p.finc = spec->fire_params[3];
    p.fdec = spec->fire_params[4];
    p.nmin = spec->nmin;
    p.mass = spec->mass;
    p.fcut = spec->fcut;
    p.max_steps = spec->nmax;
    p.criterion = criterion;
    p.precision = precision;
    FILE *log_file = fopen(log_name, "w");
    FILE *edata_file = fopen(edata_name, "w");
    std::vector<double> pos(2 * (size_t)n_points);
    int disp_count = 1;
    int worst = NR_OK;
    auto relax = [&](double xd, double yd, nr_report &rep) -> int {
        int r = nr_affine_displace(net, miny, range, xd, yd, nullptr);
        if (r != NR_OK) return r;
        r = nr_relax(net, &p, &rep, nullptr);
        if (r < 0) return r;
        if (r == NR_NOT_CONVERGED) worst = NR_NOT_CONVERGED;
        const double measure = criterion == NR_CRIT_MAX ? rep.max_force : rep.rms_force;
        if (log_file) {
            fprintf(log_file, measure <= spec->fcut ? "Convergence reached: " : "Convergence not reached: ");
            fprintf(log_file, "Steps: %d, RMS Force: %12.8le\n", rep.steps, rep.rms_force);
        }
        printf("Steps: %d, RMS Force: %12.8le\n", rep.steps, rep.rms_force);
        return NR_OK;
    };
    double min_disp = spec->compr[0] * smult, max_disp = spec->compr[1] * smult, inc = spec->compr[2] * smult;
    double curr_disp = 0.0;
    if (max_disp > 0) {
        for (curr_disp = min_disp; curr_disp <= max_disp + 1e-10; curr_disp += inc) {
            nr_report rep;
            rc = relax(0, -inc, rep);
            if (rc < 0) break;
            if (edata_file) {
                fprintf(edata_file, "%12.0lf\t%12.10lf\t%12.8le\t%12.8le\t%12.8le", 0., curr_disp, rep.e_stretch,
                        rep.e_bend, rep.e_stretch + rep.e_bend);
                if (spec->stress_columns) fprintf(edata_file, "\t%12.8le\t%12.8le", rep.stress_xy, rep.stress_yy);
                fputc('\n', edata_file);
            }
            if (!(inc > 0)) break;
        }
    }
    const double max_comp = max_disp > min_disp ? curr_disp - inc : max_disp;
    min_disp = spec->shear[0] * smult;
    max_disp = spec->shear[1] * smult;
    inc = spec->shear[2] * smult;
    if (rc >= 0 && max_disp > 0) {
        for (curr_disp = min_disp; curr_disp <= max_disp + 1e-10; curr_disp += inc) {
            nr_report rep;
            rc = relax(inc, 0, rep);
            if (rc < 0) break;
            if (edata_file) {
                fprintf(edata_file, "%12.10lf\t%12.10lf\t%12.10le\t%12.10le\t%12.10le", curr_disp, max_comp,
                        rep.e_stretch, rep.e_bend, rep.e_stretch + rep.e_bend);
                if (spec->stress_columns) fprintf(edata_file, "\t%12.10le\t%12.10le", rep.stress_xy, rep.stress_yy);
                fputc('\n', edata_file);
            }
            rc = nr_network_get_positions(net, pos.data(), nullptr);
            if (rc != NR_OK) break;
            nr::write_xy_file(report_name(disp_base, num_digits, disp_count++, "pos"), pos.data(), n_points);
            if (!(inc > 0)) break;
        }
    }
    const clock_t ct = clock() - ct0;
    if (log_file) {
        fprintf(log_file, "Elapsed time: %f seconds\n", ((float)ct) / CLOCKS_PER_SEC);
        fclose(log_file);
    }
    if (edata_file) fclose(edata_file);
    nr_network_destroy(net);
    if (rc < 0) {
        fprintf(stderr, "Relaxation failed: %s\n", nr_last_error());
        return rc;
    }
    return worst;
}

/* do_relaxation_run of network_mesh_relax.cu:1095-1390 on one .nmc file:
 * the period scaled by sqrt(1 + dilation) before get_triples, the gel's
 * inverse matrices from the undilated positions, dilation, the preferred
 * dilation (printed as the reference prints it), then the compression and
 * shear loops with the gel acting when bmod > 0.  FP64 path. */
int nr_do_mesh_relaxation_run(const char *net_file, const char *log_name, const char *edata_name,
                              const char *disp_base, const nr_mesh_batch_spec *mspec, int criterion) {
    if (!net_file || !log_name || !edata_name || !disp_base || !mspec)
        return fail(NR_ERR_INVALID, "nr_do_mesh_relaxation_run: null argument");
    const nr_batch_spec *spec = &mspec->net;
    const clock_t ct0 = clock();
    nr_host_network *hn = nullptr;
    int rc = nr_read_network_mesh(net_file, &hn);
    if (rc != NR_OK) {
        fprintf(stderr, "%s: %s\n", net_file, nr_last_error());
        nr_host_network_free(hn);
        return rc;
    }
    const double area = (hn->maxx - hn->minx) * (hn->maxy - hn->miny);
    const double swell = std::sqrt(1 + mspec->dilation);
    nr_host_network_set_offset(hn, hn->offset * swell);
    if (spec->kb > 0) nr_get_triples(hn);
    const double miny = hn->miny;
    double range = (hn->maxy - hn->miny) * swell;
    const double smult = spec->absolute ? 1.0 : range;
    const double s_inc = spec->shear[2];
    const int num_digits =
        get_dec_digits(1 + (s_inc > 0 ? (int)((spec->shear[1] - spec->shear[0]) / s_inc) : 0));
    nr_network *net = nullptr;
    rc = nr_network_create(hn, spec->ks, spec->kb, nullptr, &net);
    const int n_points = hn->n_points;
    nr_host_network_free(hn);
    if (rc != NR_OK) return rc;
    double pref_d = 0;
    rc = nr_mesh_prepare(net, mspec->smod, mspec->bmod, mspec->dilation, area, &pref_d, nullptr);
    if (rc != NR_OK) {
        nr_network_destroy(net);
        return rc;
    }
    printf("Preferred dilation: %g\n", pref_d);
    nr_fire_params p;
    p.alpha0 = spec->fire_params[0];
    p.falpha = spec->fire_params[1];
    p.dt_max = spec->fire_params[2];
    p.finc = spec->fire_params[3];
    p.fdec = spec->fire_params[4];
    p.nmin = spec->nmin;
    p.mass = spec->mass;
    p.fcut = spec->fcut;
    p.max_steps = spec->nmax;
    p.criterion = criterion;
    p.precision = NR_FP64;
    FILE *log_file = fopen(log_name, "w");
    FILE *edata_file = fopen(edata_name, "w");
    std::vector<double> pos(2 * (size_t)n_points);
    int disp_count = 1;
    int worst = NR_OK;
    auto relax = [&](nr_report &rep) -> int {
        int r = nr_relax(net, &p, &rep, nullptr);
        if (r < 0) return r;
        if (r == NR_NOT_CONVERGED) worst = NR_NOT_CONVERGED;
        const double measure = criterion == NR_CRIT_MAX ? rep.max_force : rep.rms_force;
        if (log_file) {
            fprintf(log_file, measure <= spec->fcut ? "Convergence reached: " : "Convergence not reached: ");
            fprintf(log_file, "Steps: %d, RMS Force: %12.8le\n", rep.steps, rep.rms_force);
        }
        printf("Steps: %d, RMS Force: %12.8le\n", rep.steps, rep.rms_force);
        return NR_OK;
    };
    double min_disp = spec->compr[0] * smult, max_disp = spec->compr[1] * smult, inc = spec->compr[2] * smult;
    double curr_disp = 0.0;
    if (max_disp > 0) {
        rc = nr_affine_displace(net, miny, range, 0, -min_disp, nullptr);
        range -= min_disp;
        for (curr_disp = min_disp; rc >= 0 && curr_disp <= max_disp + 1e-10; curr_disp += inc) {
            nr_report rep;
            rc = relax(rep);
            if (rc < 0) break;
            if (edata_file)
                fprintf(edata_file, "%12.0lf\t%12.10lf\t%12.8le\t%12.8le\t%12.8le\t%12.8le\n", 0., curr_disp,
                        rep.e_stretch, rep.e_bend, rep.e_gel, rep.e_stretch + rep.e_bend + rep.e_gel);
            if (curr_disp < max_disp) {
                rc = nr_affine_displace(net, miny, range, 0, -inc, nullptr);
                range -= inc;
            }
            if (!(inc > 0)) break;
        }
    }
    const double max_comp = max_disp > min_disp ? curr_disp - inc : max_disp;
    min_disp = spec->shear[0] * smult;
    max_disp = spec->shear[1] * smult;
    inc = spec->shear[2] * smult;
    if (rc >= 0 && max_disp > 0) {
        rc = nr_affine_displace(net, miny, range, min_disp, 0, nullptr);
        for (curr_disp = min_disp; rc >= 0 && curr_disp <= max_disp + 1e-10; curr_disp += inc) {
            nr_report rep;
            rc = relax(rep);
            if (rc < 0) break;
            if (edata_file)
                fprintf(edata_file, "%12.8lf\t%12.8lf\t%12.8le\t%12.8le\t%12.8le\t%12.8le\n", curr_disp, max_comp,
                        rep.e_stretch, rep.e_bend, rep.e_gel, rep.e_stretch + rep.e_bend + rep.e_gel);
            rc = nr_network_get_positions(net, pos.data(), nullptr);
            if (rc != NR_OK) break;
            nr::write_xy_file(report_name(disp_base, num_digits, disp_count++, "pos"), pos.data(), n_points);
            if (curr_disp < max_disp) rc = nr_affine_displace(net, miny, range, inc, 0, nullptr);
            if (!(inc > 0)) break;
        }
    }
    const clock_t ct = clock() - ct0;
    if (log_file) {
        fprintf(log_file, "Elapsed time: %f seconds\n", ((float)ct) / CLOCKS_PER_SEC);
        fclose(log_file);
    }
    if (edata_file) fclose(edata_file);
    nr_network_destroy(net);
    if (rc < 0) {
        fprintf(stderr, "Relaxation failed: %s\n", nr_last_error());
        return rc;
    }
    return worst;
}

}  // extern "C"

static int relaxation_batch(const char *batch_file, int precision, int criterion, int absolute, bool mesh,
                            int stress_columns = 0) {
    nr_mesh_batch_spec mspec;
    int rc = mesh ? nr_parse_mesh_batch_file(batch_file, &mspec) : nr_parse_batch_file(batch_file, &mspec.net);
    nr_batch_spec &spec = mspec.net;
    spec.absolute = absolute;
    spec.stress_columns = stress_columns;
    if (rc != NR_OK) {
        fprintf(stderr, "Parsing of the batch file failed.\n");
        return rc;
    }
    FileLists fl;
    if (!file_lists(spec.base, mesh ? "nmc" : "dat", spec.tag, fl)) {
        fprintf(stderr, "File lists could not be read.\n");
        return fail(NR_ERR_IO, "file lists could not be read");
    }
    int worst = NR_OK;
    for (size_t i = 0; i < fl.dat.size(); ++i) {
        rc = mesh ? nr_do_mesh_relaxation_run(fl.dat[i].c_str(), fl.log[i].c_str(), fl.edat[i].c_str(),
                                              fl.disp[i].c_str(), &mspec, criterion)
                  : nr_do_relaxation_run(fl.dat[i].c_str(), fl.log[i].c_str(), fl.edat[i].c_str(), fl.disp[i].c_str(),
                                         &spec, precision, criterion);
        if (rc < 0) worst = rc;
        else if (rc == NR_NOT_CONVERGED && worst == NR_OK) worst = rc;
    }
    return worst;
}

/* The reference's getopt(3) loops (large_strain_relax.cu:1055,
 * network_mesh_relax.cu:1432, sparse_relax.cpp:1177) with their option
 * strings, scanned without getopt's global state: options may be grouped
 * ("-ib f"), an argument attached ("-bfile") or in the next word (taken
 * even if it starts with '-'), "--" ends the options, and other words are
 * skipped (getopt moves them to the end, where the reference ignores
 * them).  opt(c, arg) gets each option (arg null when a required argument
 * is missing; c = '?' and arg = the character for an unknown one);
 * long_opt(name, value) gets "--name=value", or "--name value" for the
 * names in long_valued: this library's additions.  A negative return from
 * either ends the scan. */
template <class Opt, class LongOpt>
static int scan_options(int argc, char **argv, const char *spec, const std::vector<std::string> &long_valued,
                        Opt opt, LongOpt long_opt) {
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        if (strcmp(a, "--") == 0) break;
        if (a[0] != '-' || a[1] == '\0') continue;
        int rc = 0;
        if (a[1] == '-') {
            std::string name = a + 2, value;
            const size_t eq = name.find('=');
            const char *v = nullptr;
            if (eq != std::string::npos) {
                value = name.substr(eq + 1);
                name.resize(eq);
                v = value.c_str();
            } else if (i + 1 < argc && std::find(long_valued.begin(), long_valued.end(), name) != long_valued.end()) {
                v = argv[++i];
            }
            rc = long_opt(name, v);
        } else {
            for (int j = 1; a[j] && rc >= 0; ++j) {
                const char c = a[j];
                const char *p = c == ':' ? nullptr : strchr(spec, c);
                if (!p) {
                    fprintf(stderr, "%s: invalid option -- '%c'\n", argv[0], c); /* getopt's own message */
                    const char unknown[2] = {c, 0};
                    rc = opt('?', unknown);
                } else if (p[1] == ':') {
                    const char *arg = a[j + 1] ? a + j + 1 : (i + 1 < argc ? argv[++i] : nullptr);
                    if (!arg) fprintf(stderr, "%s: option requires an argument -- '%c'\n", argv[0], c);
                    rc = opt(c, arg);
                    break;
                } else {
                    rc = opt(c, nullptr);
                }
            }
        }
        if (rc < 0) return rc;
    }
    return 0;
}

static int unknown_option(const char *c) {
    if (isprint((unsigned char)c[0])) fprintf(stderr, "Unrecognized option: %c\n", c[0]);
    else fprintf(stderr, "Unknown option character.\n");
    return 0;
}

/* Both command lines: -b batch [-x bx] [-y by] [-a] [-i] (as the
 * reference's, except that -a works: there it falls through into -b and
 * copies a null optarg), plus --precision fp64|mixed, --criterion rms|max
 * and (lsrelax) --stress. */
static int cli_main(int argc, char **argv, bool mesh) {
    const char *batch_file = nullptr;
    int precision = NR_FP64, criterion = NR_CRIT_RMS, absolute = 0, stress_columns = 0;
    const int rc0 = scan_options(
        argc, argv, "ab:ix:y:", {"precision", "criterion"},
        [&](char c, const char *arg) -> int {
            switch (c) {
            case 'a': absolute = 1; return 0;
            case 'i': return 0; /* itemize: accepted and unused, as in the reference */
            case 'b':
                if (!arg) {
                    fprintf(stderr, "Option \"b\" requires a file name.\n");
                    return -1;
                }
                batch_file = arg;
                return 0;
            case 'x':
            case 'y': {
                int v = 0;
                if (!arg) {
                    fprintf(stderr, "Option \"%c\" requires a block dimension.\n", c);
                    /* the reference's else-if chain reports a missing x twice */
                    if (c == 'x') fprintf(stderr, "Unrecognized option: x\n");
                }
                else if (sscanf(arg, "%d", &v) < 1) fprintf(stderr, "Option \"%c\" requires an integer.\n", c);
                else if (v < 1) fprintf(stderr, "Block dimensions must be positive.\n");
                else printf("Block %c dimension: %d\n", c, v);
                return 0;
            }
            default: return unknown_option(arg);
            }
        },
        [&](const std::string &name, const char *v) -> int {
            if (name == "stress" && !mesh) {
                stress_columns = 1;
                return 0;
            }
            if (name != "precision" && name != "criterion") {
                fprintf(stderr, "Unrecognized option: --%s\n", name.c_str());
                return 0;
            }
            if (!v) {
                fprintf(stderr, "Option \"%s\" requires %s.\n", name.c_str(),
                        name == "precision" ? "fp64 or mixed" : "rms or max");
                return -1;
            }
            if (name == "precision") precision = strcmp(v, "mixed") == 0 ? NR_MIXED : NR_FP64;
            else criterion = strcmp(v, "max") == 0 ? NR_CRIT_MAX : NR_CRIT_RMS;
            return 0;
        });
    if (rc0 < 0) return -1;
    if (!batch_file) {
        fprintf(stderr, "No batch file was specified.\n");
        return -1;
    }
    const int rc = relaxation_batch(batch_file, precision, criterion, absolute, mesh, stress_columns);
    return rc < 0 ? 1 : 0;
}

extern "C" {

int nr_relaxation_batch(const char *batch_file, int precision, int criterion) {
    return relaxation_batch(batch_file, precision, criterion, 0, false);
}

/* parse_batch_file of sparse_relax.cpp:931-1037: blank and '#' lines are
 * skipped before each of the four entries; the file must not end right
 * after any of the first three. */
int nr_parse_spr_batch_file(const char *path, nr_spr_spec *spec) {
    if (!path || !spec) return fail(NR_ERR_INVALID, "nr_parse_spr_batch_file: null argument");
    memset(spec, 0, sizeof(*spec));
    std::ifstream input(path);
    if (!input.is_open()) {
        fprintf(stderr, "The file %s could not be read.\n", path);
        return fail(NR_ERR_IO, std::string("cannot open ") + path);
    }
    std::string line;
    auto next = [&](std::string &out) -> bool { /* next non-blank, non-comment line */
        while (!input.eof()) {
            std::getline(input, out);
            if (out.empty() || out[0] == '#') continue;
            return true;
        }
        return false;
    };
    bool got = false;
    while (next(line)) {
        std::vector<std::string> tok = split_ws(line);
        if (!tok.empty()) {
            snprintf(spec->base, sizeof(spec->base), "%s", tok[0].c_str());
            if (tok.size() > 1) snprintf(spec->tag, sizeof(spec->tag), "%s", tok[1].c_str());
            got = true;
            break;
        }
    }
    if (!got || input.eof()) {
        fprintf(stderr, "Not enough information was found.\n");
        return fail(NR_ERR_PARSE, "batch file: missing base name");
    }
    if (next(line) && (sscanf(line.c_str(), "%lf %lf %lf", &spec->ks, &spec->kb, &spec->mu) < 3 || spec->ks < 0 ||
                       spec->kb < 0 || spec->mu < 0)) {
        fprintf(stderr, "Error: invalid format for mechanical attributes.");
        return fail(NR_ERR_PARSE, "batch file: invalid mechanical attributes");
    }
    for (int which = 0; which < 2; ++which) {
        if (input.eof()) {
            fprintf(stderr, "Not enough information was provided in the batch file.\n");
            return fail(NR_ERR_PARSE, "batch file: truncated");
        }
        double *r = which == 0 ? spec->compr : spec->shear;
        if (!next(line)) return fail(NR_ERR_PARSE, "batch file: missing strain range");
        if (sscanf(line.c_str(), "%lf %lf %lf", &r[0], &r[1], &r[2]) < 3 || r[0] < 0 || r[1] < 0 || r[2] < 0 ||
            r[1] < r[0]) {
            fprintf(stderr, which == 0 ? "Error: invalid specification of compression."
                                       : "Error: invalid format for mechanical attributes.");
            return fail(NR_ERR_PARSE, "batch file: invalid strain range");
        }
    }
    return NR_OK;
}

/* do_relaxation_run of sparse_relax.cpp:676-870. */
int nr_spr_do_relaxation_run(const char *dat_name, const char *log_name, const char *disp_base, const char *e_name,
                             const nr_spr_spec *spec, int strain_mode, int affine, int itemize) {
    if (!dat_name || !spec) return fail(NR_ERR_INVALID, "nr_spr_do_relaxation_run: null argument");
    FILE *log = (log_name && log_name[0]) ? fopen(log_name, "w") : nullptr;
    const time_t start = time(nullptr);
    nr_host_network *hn = nullptr;
    int rc = nr_read_network(dat_name, &hn);
    if (rc != NR_OK) {
        fprintf(stderr, "A properly formatted network description could not be read.\n");
        nr_host_network_free(hn);
        if (log) fclose(log);
        return rc;
    }
    nr_spr *spr = nullptr;
    rc = nr_spr_create(hn, spec->ks, spec->kb, spec->mu, nullptr, &spr);
    const int n = hn->n_points;
    nr_host_network_free(hn);
    if (rc != NR_OK) {
        if (log) fclose(log);
        return rc;
    }
    nr_spr_info_t info;
    nr_spr_info(spr, &info);
    double min_c = spec->compr[0], max_c = spec->compr[1], c_inc = spec->compr[2];
    double min_s = spec->shear[0], max_s = spec->shear[1], s_inc = spec->shear[2];
    if (strain_mode) { /* :728-737: the shear is scaled by the width */
        min_c *= (info.maxy - info.miny);
        max_c *= (info.maxy - info.miny);
        c_inc *= (info.maxy - info.miny);
        if (c_inc != c_inc) c_inc = FLT_MAX - max_c;
        min_s *= (info.maxx - info.minx);
        max_s *= (info.maxx - info.minx);
        s_inc *= (info.maxx - info.minx);
        if (s_inc != s_inc) s_inc = FLT_MAX - max_c;
    }
    const bool write_disps = disp_base && disp_base[0];
    int disp_count = 1, num_digits = 1;
    if (write_disps) num_digits = get_dec_digits(2 + (int)((max_c - min_c) / c_inc) + (int)((max_s - min_s) / s_inc));
    FILE *efile = (e_name && e_name[0]) ? fopen(e_name, "w") : nullptr;
    const int max_iter = std::max(1000, std::min(10 * info.n_free_dofs, 10000000));
    rc = nr_spr_solve(spr, affine, 1e-12, max_iter, nullptr);
    int worst = rc;
    std::vector<double> u(2 * (size_t)n);
    double compression = min_c;
    while (rc >= 0 && compression < max_c + 1e-10) {
        double shear = min_s;
        while (shear < max_s + 1e-10) {
            nr_spr_record rec;
            rc = nr_spr_point(spr, compression, shear, &rec, write_disps ? u.data() : nullptr, nullptr);
            if (rc < 0) break;
            if (write_disps) {
                nr::write_xy_file(report_name(disp_base, num_digits, disp_count++, "disp"), u.data(), n);
            }
            FILE *lf = log ? log : stdout;
            fprintf(lf, "Residual RMS force: %2.10le\n", rec.residual);
            FILE *ef = efile ? efile : stdout;
            if (!itemize) fprintf(ef, "%12.8lf\t%12.8lf\t%12.10le\n", compression, shear, rec.e_total);
            else fprintf(ef, "%12.8lf\t%12.8lf\t%12.10le\t%12.10le\n", compression, shear, rec.e_ss, rec.e_bend);
            if (!(s_inc > 0)) break; /* the reference loops forever when an increment is 0 */
            shear += s_inc;
        }
        if (!(c_inc > 0)) break;
        compression += c_inc;
    }
    nr_spr_destroy(spr);
    if (efile) fclose(efile);
    if (log) {
        fprintf(log, "Elapsed time: %d seconds.\n", (int)difftime(time(nullptr), start));
        fclose(log);
    }
    if (rc < 0) {
        fprintf(stderr, "Linear solve failed: %s\n", nr_last_error());
        return rc;
    }
    return worst;
}

/* run_relaxation_batch of sparse_relax.cpp:1042-1093. */
int nr_spr_relaxation_batch(const char *batch_file, int strain_mode, int affine, int itemize) {
    nr_spr_spec spec;
    int rc = nr_parse_spr_batch_file(batch_file, &spec);
    if (rc != NR_OK) {
        fprintf(stderr, "File parsing failed.\n");
        return rc;
    }
    FileLists fl;
    if (!file_lists(spec.base, "dat", spec.tag, fl)) {
        fprintf(stderr, "File lists could not be read.\n");
        return fail(NR_ERR_IO, "file lists could not be read");
    }
    if (spec.shear[1] - spec.shear[0] < 1e-10) spec.shear[2] = 1e12;
    if (spec.compr[1] - spec.compr[0] < 1e-10) spec.compr[2] = 1e12;
    int worst = NR_OK;
    for (size_t i = 0; i < fl.dat.size(); ++i) {
        /* argument order of the reference: dat, log, disp, edata */
        rc = nr_spr_do_relaxation_run(fl.dat[i].c_str(), fl.log[i].c_str(), fl.disp[i].c_str(), fl.edat[i].c_str(),
                                      &spec, strain_mode, affine, itemize);
        if (rc < 0) worst = rc;
        else if (rc == NR_NOT_CONVERGED && worst == NR_OK) worst = rc;
    }
    return worst;
}

/* main of sparse_relax.cpp:1165-1232 (getopt "b:ginsz"); the interactive
 * mode (no -b) is not provided. */
int nr_sp_relax_main(int argc, char **argv) {
    const char *batch_file = nullptr;
    int strain_mode = 0, affine = 1, itemize = 0;
    const int rc0 = scan_options(
        argc, argv, "b:ginsz", {},
        [&](char c, const char *arg) -> int {
            switch (c) {
            case 'b':
                if (!arg) {
                    fprintf(stderr, "Option \"b\" requires a file name.\n");
                    return -1;
                }
                batch_file = arg;
                return 0;
            case 's': strain_mode = 1; return 0;
            case 'z': affine = 0; return 0;
            case 'i': itemize = 1; return 0;
            case 'g':
            case 'n': return 0; /* accepted: the solve runs on the GPU, and CG's solution has no null-space part */
            default: return unknown_option(arg);
            }
        },
        [&](const std::string &name, const char *) -> int {
            fprintf(stderr, "Unrecognized option: --%s\n", name.c_str());
            return 0;
        });
    if (rc0 < 0) return -1;
    if (!batch_file) {
        fprintf(stderr, "Only batch mode (-b) is provided.\n");
        return -1;
    }
    const int rc = nr_spr_relaxation_batch(batch_file, strain_mode, affine, itemize);
    return rc < 0 ? 1 : 0;
}

int nr_mesh_relaxation_batch(const char *batch_file, int criterion) {
    return relaxation_batch(batch_file, NR_FP64, criterion, 0, true);
}

int nr_lsrelax_main(int argc, char **argv) { return cli_main(argc, argv, false); }

int nr_nmrelax_main(int argc, char **argv) { return cli_main(argc, argv, true); }

}  // extern "C"
