// Host-side reader of GeoFLAC .inp parameter files.
//
// Restates src/read_params.f90:3-373: the same read order, the same
// list-directed value semantics (values separated by blanks or commas, a
// record may continue onto the next line, what is left of a record after the
// last value is discarded, `r*c` repeat counts, `/` ends a read), and the same
// comment rule: AdvanceToNextInputLine (read_params.f90:351-373) skips lines
// whose first character is ';'.  Text after a ';' inside a data line is
// ignored (the reference's inputs use it for trailing remarks).

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/geoflac_gb300.h"

namespace {

struct ParseError {
    int line;
    std::string what;
};

class ListReader {
  public:
    explicit ListReader(std::vector<std::string> lines) : lines_(std::move(lines)) {}

    // AdvanceToNextInputLine: skip records whose first character is ';'.
    void advance() {
        while (cur_ < lines_.size() && !lines_[cur_].empty() && lines_[cur_][0] == ';') ++cur_;
        if (cur_ >= lines_.size()) throw ParseError{(int)cur_ + 1, "end of file"};
    }

    // One list-directed READ statement: begin(), values, end().
    void begin() {
        if (cur_ >= lines_.size()) throw ParseError{(int)cur_ + 1, "end of file"};
        load(cur_);
        in_read_ = true;
        slashed_ = false;
        repeat_left_ = 0;
    }
    void end() {
        // the rest of the current record is discarded
        ++cur_;
        in_read_ = false;
    }
    // A READ with an empty item list consumes exactly one record.
    void skip_record() {
        begin();
        end();
    }

    bool next_int(int &v) {
        std::string t;
        if (!next_token(t)) return false;
        char *e = nullptr;
        errno = 0;
        long x = std::strtol(t.c_str(), &e, 10);
        if (e == t.c_str() || *e != '\0' || errno) throw ParseError{(int)cur_ + 1, "bad integer '" + t + "'"};
        v = (int)x;
        return true;
    }
    bool next_real(double &v) {
        std::string t;
        if (!next_token(t)) return false;
        for (auto &ch : t)
            if (ch == 'd' || ch == 'D') ch = 'e';
        char *e = nullptr;
        errno = 0;
        double x = std::strtod(t.c_str(), &e);
        if (e == t.c_str() || *e != '\0') throw ParseError{(int)cur_ + 1, "bad real '" + t + "'"};
        v = x;
        return true;
    }
    bool next_string(char *dst, size_t cap) {
        std::string t;
        if (!next_token(t)) return false;
        std::snprintf(dst, cap, "%s", t.c_str());
        return true;
    }
    int line() const { return (int)cur_ + 1; }

  private:
    // Split one record into raw items; "" marks a null value (two commas).
    void load(size_t idx) {
        items_.clear();
        pos_ = 0;
        std::string s = lines_[idx];
        // a ';' inside a data line starts a trailing remark
        size_t sc = s.find(';');
        if (sc != std::string::npos) s = s.substr(0, sc);
        size_t i = 0, n = s.size();
        bool last_was_comma = true; // a leading comma yields a null value
        while (i < n) {
            char ch = s[i];
            if (ch == ' ' || ch == '\t' || ch == '\r') {
                ++i;
                continue;
            }
            if (ch == ',') {
                if (last_was_comma) items_.push_back(std::string("\x01")); // null
                last_was_comma = true;
                ++i;
                continue;
            }
            if (ch == '/') {
                items_.push_back(std::string("/"));
                break;
            }
            std::string tok;
            if (ch == '\'' || ch == '"') {
                char q = ch;
                ++i;
                while (i < n && s[i] != q) tok += s[i++];
                ++i;
            } else {
                while (i < n && s[i] != ' ' && s[i] != '\t' && s[i] != ',' && s[i] != '\r' && s[i] != '/')
                    tok += s[i++];
            }
            items_.push_back(tok);
            last_was_comma = false;
        }
    }

    // Returns false when the value is null or the read was ended by '/'.
    bool next_token(std::string &out) {
        if (slashed_) return false;
        if (repeat_left_ > 0) {
            --repeat_left_;
            if (repeat_null_) return false;
            out = repeat_val_;
            return true;
        }
        while (pos_ >= items_.size()) {
            // list-directed input continues on the next record
            ++cur_;
            if (cur_ >= lines_.size()) throw ParseError{(int)cur_ + 1, "end of file inside a record"};
            load(cur_);
        }
        std::string t = items_[pos_++];
        if (t == "/") {
            slashed_ = true;
            return false;
        }
        if (t == "\x01") return false;
        size_t star = t.find('*');
        if (star != std::string::npos && star > 0 && t.find_first_not_of("0123456789") == star) {
            int r = std::atoi(t.substr(0, star).c_str());
            std::string rest = t.substr(star + 1);
            repeat_null_ = rest.empty();
            repeat_val_ = rest;
            repeat_left_ = r - 1;
            if (repeat_null_) return false;
            out = rest;
            return true;
        }
        out = t;
        return true;
    }

    std::vector<std::string> lines_;
    size_t cur_ = 0;
    std::vector<std::string> items_;
    size_t pos_ = 0;
    bool in_read_ = false, slashed_ = false;
    int repeat_left_ = 0;
    bool repeat_null_ = false;
    std::string repeat_val_;
};

void parse(ListReader &r, gf_params *p) {
    int idum;
    // ---- MESH (read_params.f90:14-75)
    r.advance();
    r.begin();
    r.next_int(p->nx);
    r.next_int(p->nz);
    r.end();
    p->nx += 1;
    p->nz += 1;
    r.advance();
    r.begin();
    r.next_real(p->x0);
    r.next_real(p->z0);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->rxbo);
    r.next_real(p->rzbo);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->ircoord);
    r.next_string(p->coordfile, sizeof p->coordfile);
    r.end();
    if (p->ircoord > 0) {
        r.advance();
        r.begin();
        r.next_int(p->nzonx);
        r.end();
        if (p->nzonx != 0) throw ParseError{r.line(), "ircoord is set, but nzonx is not 0"};
        r.advance();
        r.begin();
        r.next_int(p->nzony);
        r.end();
        if (p->nzony != 0) throw ParseError{r.line(), "ircoord is set, but nzony is not 0"};
    } else {
        r.advance();
        r.begin();
        r.next_int(p->nzonx);
        r.end();
        if (p->nzonx == 0) {
            p->nzonx = 1;
            p->nelz_x[0] = p->nx - 1;
            p->sizez_x[0] = 1.0;
        } else {
            if (p->nzonx > GF_MAXZONE) throw ParseError{r.line(), "too many x zones"};
            for (int i = 0; i < p->nzonx; ++i) {
                r.advance();
                r.begin();
                r.next_int(p->nelz_x[i]);
                r.next_real(p->sizez_x[i]);
                r.end();
            }
        }
        r.advance();
        r.begin();
        r.next_int(p->nzony);
        r.end();
        if (p->nzony == 0) {
            p->nzony = 1;
            p->nelz_y[0] = p->nz - 1;
            p->sizez_y[0] = 1.0;
        } else {
            if (p->nzony > GF_MAXZONE) throw ParseError{r.line(), "too many z zones"};
            for (int i = 0; i < p->nzony; ++i) {
                p->sizez_y[i] = 1.0;
                r.advance();
                r.begin();
                r.next_int(p->nelz_y[i]);
                r.next_real(p->sizez_y[i]);
                r.end();
            }
        }
    }
    // ---- MECHANICAL CONDITIONS (read_params.f90:77-99)
    r.advance();
    r.begin();
    r.next_int(p->nystressbc);
    r.next_int(p->nydrsides);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->nofbc);
    r.end();
    if (p->nofbc > GF_MAXBC) throw ParseError{r.line(), "too many boundary conditions"};
    r.advance(); // once, before the loop (read_params.f90:84)
    for (int i = 0; i < p->nofbc; ++i) {
        r.begin();
        r.next_int(p->nofside[i]);
        r.next_int(p->nbc1[i]);
        r.next_int(p->nbc2[i]);
        r.next_int(p->nbc[i]);
        r.next_real(p->bca[i]);
        r.next_real(p->bcb[i]);
        r.next_real(p->bcc[i]);
        r.next_real(p->bcd[i]);
        r.next_real(p->bce[i]);
        r.next_real(p->bcf[i]);
        r.next_real(p->bcg[i]);
        r.next_real(p->bch[i]);
        r.next_real(p->bci[i]);
        r.end();
    }
    r.advance();
    r.advance();
    r.begin();
    r.next_int(p->nyhydro);
    r.next_real(p->pisos);
    r.next_int(p->iphsub);
    r.next_real(p->drosub);
    r.next_real(p->damp_vis);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->g);
    r.end();
    // ---- THERMAL CONDITIONS (read_params.f90:103-187)
    r.advance();
    r.begin();
    r.next_int(p->i_prestress);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->extra_pres);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->itherm);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->istress_therm);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->ishearh);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->t_top);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->t_bot);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->hs);
    r.next_real(p->hr);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->itemp_bc);
    r.next_real(p->bot_bc);
    r.end();
    if (p->itemp_bc == 2) p->bot_bc = p->bot_bc / 1000;
    r.advance();
    r.begin();
    r.next_int(p->irtemp);
    r.end();
    if (p->irtemp > 0) {
        r.advance();
        r.begin();
        r.next_string(p->tempfile, sizeof p->tempfile);
        r.end();
    } else {
        r.advance();
        r.skip_record();
    }
    r.advance();
    r.begin();
    r.next_int(p->nzone_age);
    r.end();
    if (p->nzone_age > GF_MAXZONE_AGE) throw ParseError{r.line(), "too many age zones"};
    r.advance();
    for (int i = 0; i < p->nzone_age; ++i) {
        r.begin();
        r.next_int(p->ictherm[i]);
        r.next_real(p->age_1[i]);
        r.next_real(p->tp1[i]);
        r.next_real(p->tp2[i]);
        r.next_int(p->ixtb1[i]);
        r.next_int(p->ixtb2[i]);
        r.end();
        r.advance();
        r.begin();
        r.next_int(p->nph_layer[i]);
        if (p->nph_layer[i] > GF_MAXZONE_LAYER || p->nph_layer[i] < 1)
            throw ParseError{r.line(), "bad nph_layer"};
        for (int j = 0; j < p->nph_layer[i] - 1; ++j) r.next_real(p->hc[i][j]);
        r.end();
        r.begin();
        for (int j = 0; j < p->nph_layer[i]; ++j) r.next_int(p->iph_col[i][j]);
        r.end();
    }
    // smooth transitions between age zones (read_params.f90:162-187)
    for (int i = 0; i < p->nzone_age - 1; ++i) {
        p->iph_col_trans[i] = 0;
        if (p->ixtb2[i] == -1) {
            p->iph_col_trans[i] = 1;
            p->ixtb2[i] = p->ixtb2[i + 1];
            p->ixtb1[i + 1] = p->ixtb1[i];
        }
    }
    // ---- RHEOLOGY (read_params.f90:189-200)
    r.advance();
    r.begin();
    r.next_int(p->nphase);
    r.end();
    if (p->nphase < 1 || p->nphase > GF_MAXPH) throw ParseError{r.line(), "bad nphase"};
    for (int i = 0; i < p->nphase; ++i) {
        r.advance();
        r.begin();
        r.next_int(p->irheol[i]);
        r.next_real(p->visc[i]);
        r.next_real(p->den[i]);
        r.next_real(p->alfa[i]);
        r.next_real(p->beta[i]);
        r.next_real(p->pln[i]);
        r.next_real(p->acoef[i]);
        r.next_real(p->eactiv[i]);
        r.next_real(p->vactiv[i]);
        r.next_real(p->rl[i]);
        r.next_real(p->rm[i]);
        r.next_real(p->plstrain1[i]);
        r.next_real(p->plstrain2[i]);
        r.next_real(p->fric1[i]);
        r.next_real(p->fric2[i]);
        r.next_real(p->cohesion1[i]);
        r.next_real(p->cohesion2[i]);
        r.next_real(p->dilat1[i]);
        r.next_real(p->dilat2[i]);
        r.next_real(p->conduct[i]);
        r.next_real(p->cp[i]);
        r.next_real(p->ts[i]);
        r.next_real(p->tl[i]);
        r.next_real(p->tk[i]);
        r.next_real(p->erodibility[i]);
        r.end();
    }
    r.advance();
    r.begin();
    r.next_int(p->irphase);
    r.end();
    if (p->irphase > 0) {
        r.advance();
        r.begin();
        r.next_string(p->phasefile, sizeof p->phasefile);
        r.end();
    } else {
        r.advance();
        r.skip_record();
    }
    // inclusions (read_params.f90:218-230)
    r.advance();
    r.begin();
    r.next_int(p->inhom);
    r.end();
    if (p->inhom > GF_MAXINH) throw ParseError{r.line(), "Read_params: Increase arrays for inhomogenities"};
    for (int i = 0; i < p->inhom; ++i) {
        r.advance();
        r.begin();
        r.next_int(p->ix1[i]);
        r.next_int(p->ix2[i]);
        r.next_int(p->iy1[i]);
        r.next_int(p->iy2[i]);
        r.next_int(p->inphase[i]);
        r.next_int(p->igeom[i]);
        r.next_real(p->xinitaps[i]);
        r.end();
    }
    r.advance();
    r.begin();
    r.next_real(p->ten_off);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->tau_heal);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->v_min);
    r.next_real(p->v_max);
    r.next_int(p->ivis_shape);
    r.next_real(p->efoldc);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->itype_melting);
    r.next_int(p->nelem_serp);
    r.next_int(p->nelem_dike);
    r.next_real(p->prod_magma);
    r.next_real(p->prod_magma2);
    r.next_real(p->rho_magma);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->angle_mzone);
    r.next_real(p->fmagma_max);
    r.next_real(p->ratio_mantle_mzone);
    r.next_real(p->ratio_crust_mzone);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->latent_heat_magma);
    r.next_real(p->lambda_freeze);
    r.next_real(p->lambda_freeze_tdep);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->weaken_ratio_plastic);
    r.next_real(p->weaken_ratio_viscous);
    r.end();
    p->weaken_ratio_viscous = std::log(p->weaken_ratio_viscous);
    // ---- REMESHING (read_params.f90:257-272)
    r.advance();
    r.begin();
    r.next_int(p->ny_rem);
    r.next_int(p->mode_rem);
    r.next_int(p->ntest_rem);
    r.next_real(p->angle_rem);
    r.end();
    if (p->mode_rem != 1 && p->mode_rem != 11 && p->mode_rem != 3 && p->mode_rem != 4)
        throw ParseError{r.line(), "Illegal remeshing mode! Allowable - 1, 3, 4or 11"};
    r.advance();
    r.begin();
    r.next_real(p->dx_rem);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->topo_kappa);
    r.next_real(p->fac_kappa);
    r.end();
    // ---- PROCESS CONTROL (read_params.f90:275-313)
    r.advance();
    r.begin();
    r.next_int(p->idt_scale);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->dt_scale);
    r.next_real(p->strain_inert);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->i_rey);
    r.next_real(p->xReyn);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->ifreq_rmasses);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->ifreq_imasses);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->ifreq_visc);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->ifreq_avgsr);
    r.end();
    if (p->ifreq_rmasses <= 0 || p->ifreq_imasses <= 0 || p->ifreq_visc <= 0 || p->ifreq_avgsr <= 0)
        throw ParseError{r.line(), "process frequencies must be positive"};
    if (p->ntest_rem % p->ifreq_rmasses + p->ntest_rem % p->ifreq_imasses + p->ntest_rem % p->ifreq_visc +
            p->ntest_rem % p->ifreq_avgsr !=
        0)
        throw ParseError{r.line(), "ntest_rem must be multiples of process frequency"};
    r.advance();
    r.begin();
    r.next_real(p->frac);
    r.next_real(p->fracm);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->movegrid);
    r.next_int(p->ndim);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->demf);
    r.next_int(p->mix_strain);
    r.next_int(p->mix_stress);
    r.end();
    // ---- OUTPUT PARAMETERS (read_params.f90:315-341)
    r.advance();
    r.begin();
    r.next_real(p->time_max);
    r.end();
    p->time_max = p->time_max * 1000 * GF_SEC_YEAR;
    r.advance();
    r.begin();
    r.next_real(p->dtout_screen);
    r.end();
    p->dtout_screen = p->dtout_screen * 1000 * GF_SEC_YEAR;
    r.advance();
    r.begin();
    r.next_real(p->dtout_file);
    r.end();
    p->dtout_file = p->dtout_file * 1000 * GF_SEC_YEAR;
    r.advance();
    r.begin();
    for (int k = 0; k < 19; ++k) r.next_int(p->io_flags[k]);
    r.end();
    r.advance();
    r.begin();
    r.next_int(p->lastout);
    r.end();
    r.advance();
    r.begin();
    r.next_real(p->dtsave_file);
    r.end();
    p->dtsave_file = p->dtsave_file * 1000 * GF_SEC_YEAR;
    r.advance();
    r.begin();
    r.next_int(p->lastsave);
    r.end();
    (void)idum;
}

} // namespace

extern "C" int gf_read_params(const char *path, gf_params *p) {
    if (!path || !p) return GF_ERR_ARG;
    std::ifstream f(path);
    if (!f) return GF_ERR_IO;
    std::vector<std::string> lines;
    std::string s;
    while (std::getline(f, s)) lines.push_back(s);
    // keep the caller's extension options, reset everything else
    int mps = p->markers_per_side, ecl = p->eclogite_rule, tsw = p->therm_sweeps;
    std::memset(p, 0, sizeof *p);
    p->markers_per_side = mps > 0 ? mps : 3;
    p->eclogite_rule = ecl;
    p->therm_sweeps = tsw;
    ListReader r(std::move(lines));
    try {
        parse(r, p);
    } catch (const ParseError &e) {
        std::fprintf(stderr, "gf_read_params: %s at line %d of %s\n", e.what.c_str(), e.line, path);
        return GF_ERR_PARSE;
    }
    if (p->nx < 2 || p->nz < 2) return GF_ERR_PARSE;
    return GF_OK;
}

extern "C" int gf_layout_sizes(const gf_params *p, size_t *n_node, size_t *n_elem, size_t *max_markers) {
    if (!p || p->nx < 2 || p->nz < 2) return GF_ERR_ARG;
    if (n_node) *n_node = (size_t)p->nx * p->nz;
    if (n_elem) *n_elem = (size_t)(p->nx - 1) * (p->nz - 1);
    // allocate_markers (marker_data.f90:27)
    if (max_markers) *max_markers = (size_t)p->nx * p->nz * GF_MAX_MARKERS_PER_ELEM;
    return GF_OK;
}

extern "C" size_t gf_struct_size(int which) {
    switch (which) {
    case 0: return sizeof(gf_params);
    case 1: return sizeof(gf_clock);
    case 2: return sizeof(gf_layout);
    default: return 0;
    }
}
