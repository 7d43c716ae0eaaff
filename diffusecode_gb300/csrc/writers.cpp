// The file writers of the output menu and of calc_hkl, on the host: the
// values come from qval (dgpu_qval) or from calc_hkl's core (dgpu_calc_hkl),
// and every record is formatted with the edit descriptors of the reference's
// FORMAT statements, restated here:
//
//   Iw / I0      right-justified integer / minimal width;
//   Fw.d / F0.d  d decimals, the leading zero dropped only when it does not
//                fit, w asterisks when the field overflows;
//   Ew.d[Ee]     0.ddddE+xx (scale factor 0), exponent E+dd up to 99 and
//                +ddd to 999 without Ee, exactly e digits with Ee;
//   Aw           the rightmost w characters right-justified / the leftmost w;
//   nX           blanks, dropped at the end of a record;
//   list-directed (WRITE(u,*)): a blank then I11 per default integer, a
//                blank then 17 significant digits in a 25-character G field
//                per REAL(8) (F20.(17-k) and 5 blanks for 0.1 <= |x| < 1e17,
//                else 1PE25.16E3), as gfortran lays them out.
//
// Rounding is round-to-nearest on the exact binary value (the C library's
// conversion), the processor's default mode for formatted output.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/discus_gpu.h"
#include "hdf5_yell.h"

namespace {

// ---------------------------------------------------------------- editing

std::string stars(int w) { return std::string((size_t)(w > 0 ? w : 0), '*'); }

std::string pad_left(const std::string &s, int w)
{
    if ((int)s.size() >= w) return s;
    return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

std::string edit_i(int w, long long v)
{
    char b[64];
    snprintf(b, sizeof b, "%lld", v);
    std::string s(b);
    return (int)s.size() > w ? stars(w) : pad_left(s, w);
}

std::string edit_i0(long long v)
{
    char b[64];
    snprintf(b, sizeof b, "%lld", v);
    return b;
}

// digits of |v| with d decimals, and the sign
std::string fixed_abs(int d, double v)
{
    std::vector<char> b(400);
    snprintf(b.data(), b.size(), "%.*f", d, fabs(v));
    return b.data();
}

std::string edit_f(int w, int d, double v)
{
    if (isnan(v)) return pad_left("NaN", w);
    if (isinf(v)) return pad_left(v < 0 ? "-Inf" : "Inf", w);
    std::string m = fixed_abs(d, v);
    const std::string sg = signbit(v) ? "-" : "";
    if ((int)(sg.size() + m.size()) > w && m.size() > 1 && m[0] == '0' && m[1] == '.') m = m.substr(1);
    const std::string s = sg + m;
    return (int)s.size() > w ? stars(w) : pad_left(s, w);
}

std::string edit_f0(int d, double v)
{
    if (isnan(v)) return "NaN";
    if (isinf(v)) return v < 0 ? "-Inf" : "Inf";
    return (signbit(v) ? "-" : "") + fixed_abs(d, v);
}

// Ew.d (e = 0) or Ew.dEe, scale factor 0: [-]0.d1..dd followed by the exponent
std::string edit_e(int w, int d, double v, int e = 0)
{
    if (isnan(v)) return pad_left("NaN", w);
    if (isinf(v)) return pad_left(v < 0 ? "-Inf" : "Inf", w);
    std::string digits;
    int x = 0;                                  // v = 0.d1d2... * 10^x
    if (v == 0.0) {
        digits.assign((size_t)d, '0');
    } else {
        char b[128];
        snprintf(b, sizeof b, "%.*e", d - 1, fabs(v));     // d1.d2...dd e+X, rounded to d digits
        const char *p = b;
        digits.push_back(*p++);
        if (*p == '.') ++p;
        while (*p && *p != 'e') digits.push_back(*p++);
        x = atoi(p + 1) + 1;
    }
    std::string ex;
    const int ax = x < 0 ? -x : x;
    char b[32];
    if (e == 0) {
        if (ax <= 99) snprintf(b, sizeof b, "E%c%02d", x < 0 ? '-' : '+', ax);
        else if (ax <= 999) snprintf(b, sizeof b, "%c%03d", x < 0 ? '-' : '+', ax);
        else return stars(w);
    } else {
        long long lim = 1;
        for (int k = 0; k < e; k++) lim *= 10;
        if (ax >= lim) return stars(w);
        snprintf(b, sizeof b, "E%c%0*d", x < 0 ? '-' : '+', e, ax);
    }
    ex = b;
    const std::string sg = signbit(v) ? "-" : "";
    std::string s = sg + "0." + digits + ex;
    if ((int)s.size() > w) s = sg + "." + digits + ex;      // the optional leading zero
    return (int)s.size() > w ? stars(w) : pad_left(s, w);
}

std::string edit_a(int w, const std::string &s)
{
    if ((int)s.size() >= w) return s.substr(0, (size_t)w);
    return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

// list-directed items (each with its leading separator)
std::string ld_int(long long v)
{
    char b[64];
    snprintf(b, sizeof b, " %11lld", v);
    return b;
}

std::string ld_real(double v)
{
    if (isnan(v)) return " " + pad_left("NaN", 25);
    if (isinf(v)) return " " + pad_left(v < 0 ? "-Infinity" : "Infinity", 25);
    char b[128];
    int x = 0;                                  // |v| rounded to 17 digits = m * 10^x, 1 <= m < 10
    if (v != 0.0) {
        snprintf(b, sizeof b, "%.16e", fabs(v));
        x = atoi(strchr(b, 'e') + 1);
    }
    if (v == 0.0 || (x >= -1 && x < 17)) {
        const int k = v == 0.0 ? 1 : x + 1;     // digits before the decimal point
        std::string m = fixed_abs(17 - k, v);
        if (v == 0.0) m = fixed_abs(16, 0.0);
        const std::string s = (signbit(v) ? "-" : "") + m;
        return " " + pad_left(s, 20) + "     ";
    }
    std::string m(b);
    const size_t ep = m.find('e');
    const int ax = x < 0 ? -x : x;
    char eb[16];
    snprintf(eb, sizeof eb, "E%c%03d", x < 0 ? '-' : '+', ax);
    const std::string s = (signbit(v) ? "-" : "") + m.substr(0, ep) + eb;
    return " " + pad_left(s, 25);
}

// ---------------------------------------------------------------- records

struct Sink {
    FILE *f = nullptr;
    bool bad = false;
    explicit Sink(const std::string &path, const char *mode = "w") { f = fopen(path.c_str(), mode); }
    ~Sink()
    {
        if (f) fclose(f);
    }
    bool ok() const { return f != nullptr && !bad; }
    void rec(const std::string &s)
    {
        if (!f) return;
        if (fwrite(s.data(), 1, s.size(), f) != s.size() || fputc('\n', f) == EOF) bad = true;
    }
    void raw(const void *p, size_t n)
    {
        if (!f) return;
        if (fwrite(p, 1, n, f) != n) bad = true;
    }
    bool close()
    {
        if (!f) return false;
        const bool good = fclose(f) == 0 && !bad;
        f = nullptr;
        return good;
    }
};

// records of a repeated group: n items per record (format reversion)
template <class Fn>
void grouped(Sink &o, int64_t count, int per_record, Fn item)
{
    std::string line;
    int in = 0;
    for (int64_t k = 0; k < count; k++) {
        line += item(k);
        if (++in == per_record) {
            o.rec(line);
            line.clear();
            in = 0;
        }
    }
    if (in > 0 || count == 0) o.rec(line);
}

// qval's array and the grid position h at (i, j, l) (1-based, out_inc order)
struct Grid {
    const dgpu_output *o;
    double at(const double *v, int i, int j, int l) const
    {
        return v[(int64_t)(i - 1) + (int64_t)o->inc[0] * ((int64_t)(j - 1) + (int64_t)o->inc[1] * (l - 1))];
    }
    // h(k) = out_eck(k,1) + out_vi(k,1) REAL(i-1) + out_vi(k,2) REAL(j-1) + out_vi(k,3) REAL(l-1)
    void h(int i, int j, int l, double hv[3], bool third = true) const
    {
        for (int k = 0; k < 3; k++) {
            hv[k] = o->eck[k] + o->vi[k] * (double)(float)(i - 1) + o->vi[3 + k] * (double)(float)(j - 1);
            if (third) hv[k] += o->vi[6 + k] * (double)(float)(l - 1);
        }
    }
};

double metric_len(const double rten[9], const double h[3])
{
    // skalpro: dot_product(h, matmul(rten, h)), rten(3,3) column-major
    double s = 0.0;
    for (int a = 0; a < 3; a++) {
        double m = 0.0;
        for (int b = 0; b < 3; b++) m += rten[a + 3 * b] * h[b];
        s += h[a] * m;
    }
    return sqrt(s);
}

const double PI_D = 3.1415926535897932384626433832795;

// (1 / (1 + 0.001 exti |F|^2 lambda^3 / sind(2 asind(0.5 lambda |h|))))^0.25
double extinction(double exti, double lambda, double qq, double dstar)
{
    const double th = 2.0 * (asin(0.5 * lambda * dstar) * (180.0 / PI_D));
    return pow(1.0 / (1.0 + 0.001 * exti * qq * qq * lambda * lambda * lambda / sin(th * (PI_D / 180.0))), 0.25);
}

// INT(h(1))**2 + INT(h(2))**2 + INT(h(3))**2 /= 0
bool not_origin(const double h[3])
{
    const long long a = (long long)h[0], b = (long long)h[1], c = (long long)h[2];
    return a * a + b * b + c * c != 0;
}

// names of qval's values (qval.f90:30-36), 17 characters each
const char *CVALUE[20] = {"undefined        ", "Intensity        ", "Amplitude        ", "Phase angle      ",
                          "Real Part        ", "Imaginary Part   ", "Random Phase     ", "S(Q)             ",
                          "F(Q)             ", "f2aver = <f^2>   ", "faver2 = <f>^2   ", "faver = <f>      ",
                          "Normal Inten     ", "I(Q)             ", "PDF              ", "3DPDF            ",
                          "3DBETA           ", "f2averb=<f^2>*DBW", "faver2b=<f>^2*DBW", "faverb = <F>     "};

std::string rtrim(std::string s)
{
    while (!s.empty() && s.back() == ' ') s.pop_back();
    return s;
}

// ------------------------------------------------------- NIPL header lines

// angle between hor and ver in the reciprocal metric (metric.f90:35-86):
// acos of the normalised product divided by rad converted to default REAL
double bang(const double rten[9], const double u[3], const double w[3])
{
    double xu[3], yw[3];
    for (int k = 0; k < 3; k++) {
        xu[k] = 0.0 - u[k];
        yw[k] = 0.0 - w[k];
    }
    auto sk = [&](const double *p, const double *q) {
        double s = 0.0;
        for (int a = 0; a < 3; a++) {
            double m = 0.0;
            for (int b = 0; b < 3; b++) m += rten[a + 3 * b] * q[b];
            s += p[a] * m;
        }
        return s;
    };
    const double xx = sqrt(sk(xu, xu)), xy = sk(xu, yw), yy = sqrt(sk(yw, yw));
    if (!(xx > 0 && yy > 0)) return 0.0;
    const double arg = xy / (xx * yy);
    if (fabs(arg) < 1.0) return acos(arg) / (double)(float)(PI_D / 180.0);
    return arg >= 1.0 ? 0.0 : 180.0;
}

// four_angles (four_angles_mod.f90:7-106): angle and aver of the pairs
// (ver, hor), (hor, top), (top, ver)
void four_angles(const dgpu_nipl *n, const double rten[9], int ea, int eo, int et, double ang[3], double avr[3])
{
    const double *hor = n->vi, *ver = n->vi + 3, *top = n->vi + 6;
    const bool ltop = !(n->eck[0] == n->eck[9] && n->eck[1] == n->eck[10] && n->eck[2] == n->eck[11]) ||
                      n->inc[2] > 1;
    double len[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; k++)
        if (n->inc[k] > 1) len[k] = metric_len(rten, n->vi + 3 * k);
    // angle(angle, inc2, inc1, ver, hor, length2, length1, extr_ord, extr_abs)
    auto pair = [&](int inc2, int inc1, const double *v, const double *h, double l2, double l1, int e_o, int e_a,
                    double &a, double &av) {
        a = 0.0;
        av = 0.0;
        if (inc1 > 1 && inc2 > 1) {
            a = bang(rten, h, v);
            if (fabs(h[e_a - 1]) > 0.0 && fabs(v[e_o - 1]) > 0.0) av = (l2 / v[e_o - 1]) / (l1 / h[e_a - 1]);
        }
    };
    pair(n->inc[1], n->inc[0], ver, hor, len[1], len[0], eo, ea, ang[0], avr[0]);
    if (ltop && n->inc[2] > 1 && len[2] > 0.0) {
        pair(n->inc[2], n->inc[0], hor, top, len[0], len[2], ea, et, ang[1], avr[1]);
        pair(n->inc[2], n->inc[1], top, ver, len[2], len[1], et, eo, ang[2], avr[2]);
    } else {
        ang[1] = ang[2] = 90.0;
        avr[1] = avr[2] = 1.0;
    }
}

// write_discus_nipl_header (discus_nipl_header.f90:5-172) for one layer
std::vector<std::string> nipl_header(const dgpu_nipl *n, const dgpu_output *o, int layer)
{
    std::vector<std::string> cry, fou;
    const int ncry = 2 + n->nscat + 1;
    cry.push_back("# CRYSTAL : lines       ;1I:: " + edit_i(8, ncry));
    cry.push_back("# CRYSTAL : no. atoms   ;3I:: " + edit_i(12, n->natoms) + ", " + edit_i(12, n->nscat) + ", " +
                  edit_i(12, n->ncatoms));
    for (int i = 0; i <= n->nscat; i++) {
        const std::string name(n->at_lis + 4 * i, 4);
        cry.push_back("# CRYSTAL : type atom   ;1C 2I 1R:: " + edit_a(5, name) + ", " + edit_i(12, i) + ", " +
                      edit_i(12, n->amount[i]) + ", " + edit_f(8, 5, n->dw[i]));
    }
    const bool four = (n->four_last < 0 ? -n->four_last : n->four_last) < 3;
    if (four) {
        static const char *RAD[3] = {"xray", "neutron", "electron"};
        static const char AX[3] = {'h', 'k', 'l'};
        double ang[3], avr[3];
        four_angles(n, o->rten, o->extr_abs, o->extr_ord, o->extr_top, ang, avr);
        const int fl = n->four_last < 0 ? -n->four_last : n->four_last;
        auto r3 = [&](const double *v) {
            return edit_f(12, 5, v[0]) + ", " + edit_f(12, 5, v[1]) + ", " + edit_f(12, 5, v[2]);
        };
        fou.push_back("# FOURIER : lines       ;1I:: " + edit_i(8, 18));
        fou.push_back("# FOURIER : type        ;1C:: " + edit_i(1, fl) +
                      (n->four_last < 0 ? "D Fourier with lots" : "D Fourier complete crystal"));
        const int rad = n->radiation >= 1 && n->radiation <= 3 ? n->radiation - 1 : 0;
        fou.push_back(std::string("# FOURIER : radiation   ;1C:: ") + RAD[rad]);
        fou.push_back("# FOURIER : wave length ;1R::" + edit_f(12, 5, n->rlambda));
        const std::string lam = n->lambda ? rtrim(n->lambda) : "";
        fou.push_back("# FOURIER : wave name   ;" + edit_i(1, lam.empty() ? 0 : 1) + "C::" + lam);
        fou.push_back(std::string("# FOURIER : adp         ;1C:: ") + (n->ldbw ? "used" : "ignored"));
        fou.push_back(std::string("# FOURIER : dispersion  ;1C:: ") + (n->ano ? "anomalous" : "ignored"));
        fou.push_back("# FOURIER : lower left  ;3R::" + r3(n->eck));
        fou.push_back("# FOURIER : lower right ;3R::" + r3(n->eck + 3));
        fou.push_back("# FOURIER : upper left  ;3R::" + r3(n->eck + 6));
        fou.push_back("# FOURIER : top   left  ;3R::" + r3(n->eck + 9));
        fou.push_back("# FOURIER : no. points  ;3I::" + edit_i(12, n->inc[0]) + ", " + edit_i(12, n->inc[1]) + ", " +
                      edit_i(12, n->inc[2]));
        fou.push_back(std::string("# FOURIER : abscissa    ;1C:: ") + AX[o->extr_abs - 1]);
        fou.push_back(std::string("# FOURIER : ordinate    ;1C:: ") + AX[o->extr_ord - 1]);
        fou.push_back(std::string("# FOURIER : top         ;1C:: ") + AX[o->extr_top - 1]);
        fou.push_back("# FOURIER : current top ;1I:: " + edit_i(12, layer));
        fou.push_back("# FOURIER : angles      ;3R::" + r3(ang));
        fou.push_back("# FOURIER : aver        ;3R::" + r3(avr));
    }
    const int nsec = four ? 2 : 1;
    const int nheader = 1 + 1 + (four ? 1 : 0) + (int)cry.size() + (int)fou.size();
    std::vector<std::string> h;
    h.push_back("# HEADER  : lines, sec  ;2I::" + edit_i(8, nheader) + ", " + edit_i(8, nsec));
    h.push_back("# HEADER  : section     ;1C::CRYSTAL");
    if (four) h.push_back("# HEADER  : section     ;1C::FOURIER");
    for (auto &s : cry) h.push_back(rtrim(s));
    for (auto &s : fou) h.push_back(rtrim(s));
    return h;
}

// -------------------------------------------------------------- writers

// output_save_file_2d (discus_s_out_file.f90:124-260): header, npkt, ranges, rows
bool save_2d(const std::string &path, const std::vector<std::string> &hdr, const double ranges[4], int n1, int n2,
             const Grid &g, const double *v, int l)
{
    Sink o(path);
    if (!o.f) return false;
    for (auto &s : hdr) o.rec(s);
    o.rec(" " + edit_i(8, n1) + " " + edit_i(8, n2));
    o.rec(" " + edit_e(12, 5, ranges[0]) + " " + edit_e(12, 5, ranges[1]) + " " + edit_e(12, 5, ranges[2]) + " " +
          edit_e(12, 5, ranges[3]));
    for (int j = 1; j <= n2; j++)
        grouped(o, n1, 5, [&](int64_t i) { return " " + edit_e(12, 5, g.at(v, (int)i + 1, j, l)); });
    o.rec("");                                       // WRITE(iff, *)
    return o.close();
}

// ityp 0 (graphic.f90:1704-1847)
int write_standard(const std::string &path, const dgpu_output *o, const double *v)
{
    const Grid g{o};
    const int *inc = o->inc;
    const int ea = o->extr_abs, eo = o->extr_ord;
    auto ECK = [&](int axis, int corner) { return o->eck[(axis - 1) + 3 * (corner - 1)]; };
    int is_axis = 0, is_dim;
    if (inc[1] == 1 && inc[2] == 1) is_axis = 1, is_dim = 1;
    else if (inc[0] == 1 && inc[2] == 1) is_axis = 2, is_dim = 1;
    else if (inc[0] == 1 && inc[1] == 1) is_axis = 3, is_dim = 1;
    else if (inc[2] == 1) is_dim = 2;
    else is_dim = 3;
    if (is_dim == 1) {
        // output_save_file_1d: x = h(extr_abs), y = qval(i, 1, 1) along the axis
        Sink f(path);
        if (!f.f) return DGPU_ERR_IO;
        int loop[3] = {1, 1, 1};
        for (int i = 1; i <= inc[is_axis - 1]; i++) {
            loop[is_axis - 1] = i;
            double h[3];
            g.h(loop[0], loop[1], loop[2], h);
            f.rec(" " + edit_e(12, 5, h[ea - 1]) + " " + edit_e(12, 5, g.at(v, i, 1, 1)));
        }
        return f.close() ? DGPU_OK : DGPU_ERR_IO;
    }
    const double ranges[4] = {ECK(ea, 1), ECK(ea, 2), ECK(eo, 1), ECK(eo, 3)};
    if (is_dim == 2) {
        const auto hdr = o->nipl ? nipl_header(o->nipl, o, 1) : std::vector<std::string>();
        return save_2d(path, hdr, ranges, inc[0], inc[1], g, v, 1) ? DGPU_OK : DGPU_ERR_IO;
    }
    for (int l = 1; l <= inc[2]; l++) {
        const auto hdr = o->nipl ? nipl_header(o->nipl, o, l) : std::vector<std::string>();
        char part[32];
        snprintf(part, sizeof part, ".PART_%04d", l);          // FORMAT(a,'.PART_',i4.4)
        if (!save_2d(rtrim(path) + part, hdr, ranges, inc[0], inc[1], g, v, l)) return DGPU_ERR_IO;
    }
    return DGPU_OK;
}

// SHELX scale out_fac (graphic.f90:1598-1702)
double shelx_scale(const dgpu_output *o, const Grid &g, const double *ampl)
{
    const int m = (int)lround(o->valmax);           // NINT
    const bool sh = o->format == DGPU_OUT_HKLF4 || o->format == DGPU_OUT_LIST5;
    if (m == -1 && sh) {
        const double a = o->f000 / o->icc[0] / o->icc[1] / o->icc[2];
        const double qq = a * a;
        double factor = (double)(long long)(log(qq) / log(10.0)) - (o->format == DGPU_OUT_HKLF4 ? 3 : 2);
        if (factor < 0) factor = 0;
        return pow(10.0, -factor);
    }
    if (m == -2 && sh) {
        double qqmax = 0.0;
        for (int l = 1; l <= o->inc[2]; l++)
            for (int j = 1; j <= o->inc[1]; j++)
                for (int i = 1; i <= o->inc[0]; i++) {
                    double h[3];
                    g.h(i, j, l, h);
                    if (not_origin(h)) {
                        const double a = g.at(ampl, i, j, l) / o->icc[0] / o->icc[1] / o->icc[2];
                        qqmax = fmax(qqmax, a * a);
                    }
                }
        double factor = (double)(long long)(log(qqmax) / log(10.0)) - 3;
        if (o->format == DGPU_OUT_HKLF4 && factor < 0) factor = 0;
        return pow(10.0, -factor);
    }
    if (o->valmax > 0.0 && sh) return o->valmax;
    return 1.0;
}

// ityp 3, 6, 7, 8, 9 (graphic.f90:1848-2109)
int write_other(const std::string &path, dgpu_output *o, const double *v, const double *ampl, const double *phase)
{
    const Grid g{o};
    const int *inc = o->inc;
    const int fmt = o->format;
    const double cells[3] = {(double)o->icc[0], (double)o->icc[1], (double)o->icc[2]};
    const double fac = shelx_scale(o, g, ampl);
    o->out_fac = fac;
    const int ima = 6 - o->extr_abs - o->extr_ord;
    Sink f(path);
    if (!f.f) return DGPU_ERR_IO;
    auto per_cell = [&](double a) { return a / cells[0] / cells[1] / cells[2]; };
    auto positive_phase = [](double p) { return p < 0.0 ? p + 360.0 : p; };
    if (inc[0] > 1 && inc[1] > 1) {
        if (fmt == DGPU_OUT_NIPL3D) {
            auto ECK = [&](int axis, int corner) { return o->eck[(axis - 1) + 3 * (corner - 1)]; };
            f.rec(ld_int(inc[0]) + ld_int(inc[1]) + ld_int(inc[2]));
            f.rec(ld_real(ECK(o->extr_abs, 1)) + ld_real(ECK(o->extr_abs, 2)) + ld_real(ECK(o->extr_ord, 1)) +
                  ld_real(ECK(o->extr_ord, 3)) + ld_real(ECK(o->extr_top, 1)) + ld_real(ECK(o->extr_top, 4)));
            // the file is closed after the first layer when out_inc(3) > 1: the
            // later layers go to the unit's default file, not to outfile
            for (int j = 1; j <= inc[1]; j++) {
                grouped(f, inc[0], 5, [&](int64_t i) { return " " + edit_e(12, 5, g.at(v, (int)i + 1, j, 1)); });
                f.rec("");
            }
        } else if (fmt == DGPU_OUT_HKLF4 || fmt == DGPU_OUT_LIST5 || fmt == DGPU_OUT_LIST9) {
            for (int l = 1; l <= inc[2]; l++)
                for (int j = 1; j <= inc[1]; j++)
                    for (int i = 1; i <= inc[0]; i++) {
                        double h[3];
                        g.h(i, j, l, h);
                        if (!not_origin(h)) continue;
                        double qq = per_cell(g.at(ampl, i, j, l));
                        const double dstar = metric_len(o->rten, h);
                        if (fmt == DGPU_OUT_HKLF4) {
                            const double ext = o->exti > 0.00001 ? extinction(o->exti, o->rlambda, qq, dstar) : 1.0;
                            const double sq = fmax(qq * sqrt(ext) * fac * 0.10, 0.01);
                            qq = (qq * ext) * (qq * ext) * fac;
                            f.rec(edit_i(4, (long long)h[0]) + edit_i(4, (long long)h[1]) + edit_i(4, (long long)h[2]) +
                                  edit_f(8, 2, qq) + edit_f(8, 2, sq));
                        } else {
                            const double ext = extinction(o->exti, o->rlambda, qq, dstar);
                            qq = (qq * ext) * fac;
                            const double sq = positive_phase(g.at(phase, i, j, l));
                            if (fmt == DGPU_OUT_LIST5)
                                f.rec(edit_i(4, (long long)h[0]) + edit_i(4, (long long)h[1]) +
                                      edit_i(4, (long long)h[2]) + edit_f(10, 2, qq) + edit_f(10, 2, qq) +
                                      edit_f(7, 2, sq));
                            else
                                f.rec(edit_f(10, 6, h[0]) + " " + edit_f(10, 6, h[1]) + " " + edit_f(10, 6, h[2]) +
                                      " " + edit_e(12, 5, qq) + " " + edit_e(12, 5, qq) + " " + edit_f(7, 2, sq));
                        }
                    }
        } else if (fmt == DGPU_OUT_GNUPLOT) {
            for (int j = 1; j <= inc[1]; j++) {
                for (int i = 1; i <= inc[0]; i++) {
                    double h[3];
                    g.h(i, j, 1, h, false);
                    f.rec(" " + edit_e(12, 5, h[o->extr_abs - 1]) + " " + edit_e(12, 5, h[o->extr_ord - 1]) + " " +
                          edit_e(12, 5, g.at(v, i, j, 1)) + " " + edit_e(12, 5, h[ima - 1]));
                }
                f.rec("");
            }
        }
    } else if ((inc[0] == 1 || inc[1] == 1) &&
               (fmt == DGPU_OUT_HKLF4 || fmt == DGPU_OUT_LIST5 || fmt == DGPU_OUT_LIST9)) {
        // 1D rows: along j when out_inc(1) = 1, else along i; SHELX formats
        // only.  Scaling by F(000) sets the routine's value to 2 (amplitude)
        // before these rows read it.
        const bool along_j = inc[0] == 1;
        if ((int)lround(o->valmax) == -1 && (fmt == DGPU_OUT_HKLF4 || fmt == DGPU_OUT_LIST5)) v = ampl;
        const int n = along_j ? inc[1] : inc[0];
        for (int t = 1; t <= n; t++) {
            const int i = along_j ? 1 : t, j = along_j ? t : 1;
            double h[3];
            g.h(i, j, 1, h, false);
            if (!not_origin(h)) continue;
            const double val = along_j ? g.at(v, 1, j, 1) : g.at(v, i, 1, 1);
            const double ph = !phase ? 0.0 : along_j ? g.at(phase, 1, j, 1) : g.at(phase, i, 1, 1);
            if (fmt == DGPU_OUT_HKLF4) {
                const double qq = per_cell(val) * fac;
                f.rec(edit_i(4, (long long)h[0]) + edit_i(4, (long long)h[1]) + edit_i(4, (long long)h[2]) +
                      edit_f(8, 2, qq) + edit_f(8, 2, sqrt(qq)));
            } else if (fmt == DGPU_OUT_LIST5) {
                const double qq = per_cell(val) * fac;
                f.rec(edit_i(4, (long long)h[0]) + edit_i(4, (long long)h[1]) + edit_i(4, (long long)h[2]) +
                      edit_f(10, 2, qq) + edit_f(10, 2, qq) + edit_f(7, 2, positive_phase(ph)));
            } else if (fmt == DGPU_OUT_LIST9) {
                const double qq = per_cell(val);
                f.rec(edit_f(10, 6, h[0]) + " " + edit_f(10, 6, h[1]) + " " + edit_f(10, 6, h[2]) + " " +
                      edit_e(12, 5, qq) + " " + edit_e(12, 5, qq) + " " + edit_f(7, 2, positive_phase(ph)));
            }
        }
    }
    return f.close() ? DGPU_OK : DGPU_ERR_IO;
}

// vtk_write (vtk_mod.f90:4-35): the dsi array, one E13.6E2 value per record
int write_vtk(const std::string &path, const dgpu_output *o, const double *dsi, int64_t n)
{
    double d[3];
    for (int k = 0; k < 3; k++)
        d[k] = sqrt(o->vi[3 * k] * o->vi[3 * k] + o->vi[3 * k + 1] * o->vi[3 * k + 1] +
                    o->vi[3 * k + 2] * o->vi[3 * k + 2]);
    Sink f(path);
    if (!f.f) return DGPU_ERR_IO;
    f.rec("# vtk DataFile Version 3.0");
    f.rec("DISCUS OUTPUT");
    f.rec("ASCII");
    f.rec("DATASET STRUCTURED_POINTS");
    f.rec("DIMENSIONS " + edit_i0(o->inc[0]) + " " + edit_i0(o->inc[1]) + " " + edit_i0(o->inc[2]));
    f.rec("ORIGIN " + edit_f0(4, o->eck[0]) + " " + edit_f0(4, o->eck[1]) + " " + edit_f0(4, o->eck[2]));
    f.rec("SPACING " + edit_f0(4, d[0]) + " " + edit_f0(4, d[1]) + " " + edit_f0(4, d[2]));
    f.rec("POINT_DATA " + edit_i0((long long)o->inc[0] * o->inc[1] * o->inc[2]));
    f.rec("SCALARS values float");
    f.rec("LOOKUP_TABLE default");
    for (int64_t k = 0; k < n; k++) f.rec(edit_e(13, 6, dsi[k], 2));
    return f.close() ? DGPU_OK : DGPU_ERR_IO;
}

// mrc_write (lib_f90/mrc_data.f90:19-139): 4-byte direct-access records,
// 1024-byte header, 3072-byte extended header, REAL(4) image (i fastest)
int write_mrc(const std::string &path, const dgpu_output *o, const double *v)
{
    const int64_t np = (int64_t)o->inc[0] * o->inc[1] * o->inc[2];
    std::vector<uint32_t> w(256 + 768, 0u);
    auto I = [&](int rec, int32_t x) { memcpy(&w[rec - 1], &x, 4); };
    auto R = [&](int rec, float x) { memcpy(&w[rec - 1], &x, 4); };
    double mn = np > 0 ? v[0] : 0.0, mx = mn, sm = 0.0;
    for (int64_t k = 0; k < np; k++) {
        mn = fmin(mn, v[k]);
        mx = fmax(mx, v[k]);
        sm += v[k];
    }
    I(1, o->inc[0]);
    I(2, o->inc[1]);
    I(3, o->inc[2]);
    I(4, 2);
    I(5, 0);                              // nxyzstart = 0 0 0 (graphic.f90:123)
    I(6, 0);
    I(7, 0);
    I(8, o->inc[0] - 1);
    I(9, o->inc[1] - 1);
    I(10, o->inc[2] - 1);
    for (int k = 0; k < 3; k++) R(11 + k, (float)o->ar[k]);
    for (int k = 0; k < 3; k++) R(14 + k, (float)o->wrez[k]);
    R(17, (float)o->extr_abs);
    R(18, (float)o->extr_ord);
    R(19, (float)o->extr_top);
    R(20, (float)mn);
    R(21, (float)mx);
    R(22, (float)(sm / (double)(o->inc[0] * o->inc[1] * o->inc[2])));
    I(23, 0);
    I(24, 3072);
    R(50, 0.0f);
    R(51, 0.0f);
    R(52, 0.0f);
    memcpy(&w[52], "MAP", 3);             // 'MAP' in a 4-byte record, the fourth byte zero
    I(54, 4 + 4 * 16 + 68 * 256);
    Sink f(path, "wb");
    if (!f.f) return DGPU_ERR_IO;
    f.raw(w.data(), w.size() * 4);
    std::vector<float> img((size_t)np);
    for (int64_t k = 0; k < np; k++) img[(size_t)k] = (float)v[k];
    f.raw(img.data(), img.size() * 4);
    return f.close() ? DGPU_OK : DGPU_ERR_IO;
}

// xplor_write (discus_xplor.f90:16-139)
int write_xplor(std::string path, const dgpu_output *o, const double *v)
{
    if (path.size() < 6 || [&] {
            std::string t = path.substr(path.size() - 6);
            for (auto &c : t) c = (char)toupper((unsigned char)c);
            return t != ".XPLOR";
        }())
        path += ".xplor";
    const Grid g{o};
    int start[3] = {1, 1, 1}, fini[3] = {o->inc[0], o->inc[1], o->inc[2]};
    if (o->lrange != 0) {
        int center[3] = {o->center[0], o->center[1], o->center[2]};
        int pixel[3] = {o->pixel[0], o->pixel[1], o->pixel[2]};
        if (o->lcenter == 0)
            for (int k = 0; k < 3; k++) {
                const float half = (float)o->inc[k] / 2.0f;          // NINT(out_inc/2.)
                const int r = (int)lroundf(half);
                center[k] = r > 1 ? r : 1;
            }
        if (o->lpixel == 0)
            for (int k = 0; k < 3; k++) pixel[k] = o->inc[k];
        if (o->lrange == 2)
            for (int k = 0; k < 3; k++) {
                const int e = (o->inc[k] + o->inc[k] % 2);
                if (o->quad[k] == 'l') {
                    pixel[k] = e / 2;
                    center[k] = e / 4 + 1;
                } else if (o->quad[k] == 'r') {
                    pixel[k] = e / 2;
                    center[k] = e / 4 + pixel[k] + 1 - o->inc[k] % 2;
                }
            }
        for (int k = 0; k < 3; k++) {
            const int m1 = pixel[k] / 2;
            const int m2 = pixel[k] % 2 == 0 ? pixel[k] / 2 - 1 : pixel[k] / 2;
            int s = center[k] - m1, e = center[k] + m2;
            s = s > 1 ? s : 1;
            e = e > 1 ? e : 1;
            start[k] = s < o->inc[k] ? s : o->inc[k];
            fini[k] = e < o->inc[k] ? e : o->inc[k];
        }
    }
    const int val = o->value >= 0 && o->value <= 19 ? o->value : 0;
    if (val == 15) return DGPU_ERR_UNSUPPORTED;             // 3DPDF: direct-space map, not this path
    Sink f(path);
    if (!f.f) return DGPU_ERR_IO;
    f.rec("");                                              // WRITE(IMRC,*)
    const std::string title = "TITLE " + rtrim(o->name ? o->name : "") + " " + CVALUE[val] + " written by DISCUS ";
    f.rec(title.size() >= 80 ? title.substr(0, 80) : title + std::string(80 - title.size(), ' '));
    std::string dims;
    for (int k = 0; k < 3; k++) {
        const int n = fini[k] - start[k] + 1;
        dims += edit_i(8, n) + edit_i(8, 1) + edit_i(8, n);
    }
    f.rec(dims);
    if (val != 14) {
        const double p[6] = {o->ar[0], o->ar[1], o->ar[2], o->wrez[0], o->wrez[1], o->wrez[2]};
        std::string s;
        for (double x : p) s += edit_e(12, 5, x);
        f.rec(s);
    }
    f.rec(edit_a(5, "  ZYX"));
    for (int l = start[2]; l <= fini[2]; l++) {
        f.rec(edit_i(8, l - start[2] + 1));
        const int ni = fini[0] - start[0] + 1, nj = fini[1] - start[1] + 1;
        grouped(f, (int64_t)ni * nj, 6, [&](int64_t k) {
            const int i = start[0] + (int)(k % ni), j = start[1] + (int)(k / ni);
            return edit_e(12, 5, g.at(v, i, j, l));
        });
    }
    f.rec(edit_i(8, -9999));
    f.rec(edit_e(12, 4, 1.0) + " " + edit_e(12, 4, 1.0));
    return f.close() ? DGPU_OK : DGPU_ERR_IO;
}

// ------------------------------------------------------------ calc_hkl files

// Fortran formatted input of one field (BLANK='NULL': blanks ignored, an
// empty field is zero; Fw.d without a decimal point implies d decimals)
bool read_field(const std::string &line, size_t pos, size_t w, int d, bool integer, double &out)
{
    std::string s;
    for (size_t k = pos; k < pos + w && k < line.size(); k++)
        if (line[k] != ' ') s.push_back(line[k]);
    if (s.empty()) {
        out = 0.0;
        return true;
    }
    char *end = nullptr;
    if (integer) {
        const long long x = strtoll(s.c_str(), &end, 10);
        if (*end) return false;
        out = (double)x;
        return true;
    }
    std::string t = s;
    for (auto &c : t)
        if (c == 'd' || c == 'D') c = 'e';
    const bool point = t.find('.') != std::string::npos;
    out = strtod(t.c_str(), &end);
    if (*end) return false;
    if (!point) {
        // implied decimal point: the mantissa's digits shifted by d
        const size_t ep = t.find_first_of("eE");
        const double mant = strtod(t.substr(0, ep).c_str(), nullptr);
        const int ex = ep == std::string::npos ? 0 : atoi(t.c_str() + ep + 1);
        out = mant * pow(10.0, (double)(ex - d));
    }
    return true;
}

std::vector<std::string> blank_tokens(const std::string &line)
{
    std::vector<std::string> t;
    size_t k = 0;
    while (k < line.size()) {
        while (k < line.size() && (line[k] == ' ' || line[k] == '\t')) k++;
        if (k >= line.size()) break;
        const size_t s = k;
        while (k < line.size() && line[k] != ' ' && line[k] != '\t') k++;
        t.push_back(line.substr(s, k - s));
    }
    return t;
}

bool read_lines(const char *path, std::vector<std::string> &lines)
{
    FILE *f = fopen(path, "r");
    if (!f) return false;
    std::string cur;
    int c;
    while ((c = fgetc(f)) != EOF) {
        if (c == '\n') {
            if (!cur.empty() && cur.back() == '\r') cur.pop_back();
            lines.push_back(cur);
            cur.clear();
        } else {
            cur.push_back((char)c);
        }
    }
    if (!cur.empty()) lines.push_back(cur);
    fclose(f);
    return true;
}

}  // namespace

extern "C" {

int dgpu_output_write(const char *path, dgpu_output *out, const double *values, const double *ampl,
                      const double *phase, int64_t nvalues)
{
    if (!path || !out) return DGPU_ERR_ARG;
    for (int k = 0; k < 3; k++)
        if (out->inc[k] < 1) return DGPU_ERR_ARG;
    if (out->extr_abs < 1 || out->extr_abs > 3 || out->extr_ord < 1 || out->extr_ord > 3 || out->extr_top < 1 ||
        out->extr_top > 3)
        return DGPU_ERR_ARG;
    const int64_t np = (int64_t)out->inc[0] * out->inc[1] * out->inc[2];
    out->out_fac = 1.0;
    const int fmt = out->format;
    const bool shelx = fmt == DGPU_OUT_HKLF4 || fmt == DGPU_OUT_LIST5 || fmt == DGPU_OUT_LIST9;
    if (fmt == DGPU_OUT_VTK) {
        if (!values || nvalues < 0) return DGPU_ERR_ARG;
        return write_vtk(path, out, values, nvalues);
    }
    if (nvalues != np) return DGPU_ERR_ARG;
    const bool two_d = out->inc[0] > 1 && out->inc[1] > 1;
    if (shelx) {
        if (!phase && fmt != DGPU_OUT_HKLF4) return DGPU_ERR_ARG;
        if (two_d && !ampl) return DGPU_ERR_ARG;
        if (!two_d && !values) return DGPU_ERR_ARG;
        if (!ampl && (int)lround(out->valmax) == -2) return DGPU_ERR_ARG;
    } else if (!values) {
        return DGPU_ERR_ARG;
    }
    switch (fmt) {
    case DGPU_OUT_STANDARD: return write_standard(path, out, values);
    case DGPU_OUT_GNUPLOT:
    case DGPU_OUT_HKLF4:
    case DGPU_OUT_LIST5:
    case DGPU_OUT_LIST9:
    case DGPU_OUT_NIPL3D: return write_other(path, out, values, ampl, phase);
    case DGPU_OUT_MRC: return write_mrc(path, out, values);
    case DGPU_OUT_HDF5: return dgpu_hdf5::write_yell(path, out, values);
    case DGPU_OUT_XPLOR: return write_xplor(path, out, values);
    default: return DGPU_ERR_UNSUPPORTED;
    }
}

int dgpu_calc_hkl_files(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *opts, const char *infile,
                        const char *calcfile, int32_t style, double scale, double exti, double rlambda)
{
    if (!ctx || !cr || !opts || !infile || !calcfile) return DGPU_ERR_ARG;
    if (style != DGPU_HKL_HKLF4 && style != DGPU_HKL_CIF) return DGPU_ERR_ARG;
    std::vector<std::string> lines;
    if (!read_lines(infile, lines)) return DGPU_ERR_IO;
    // the reflections (fourier_sup.f90:3317-3404)
    std::vector<int32_t> hkl;
    std::vector<double> iobs;                  // HKLF4: rint; CIF: the row's values
    std::vector<std::vector<double>> rows;
    size_t nentries = 0;
    int j_icalc = 0;
    if (style == DGPU_HKL_HKLF4) {
        for (auto &ln : lines) {
            if (!ln.empty() && (ln[0] == '#' || ln[0] == '!' || ln[0] == 'd')) return DGPU_ERR_ARG;
            double v[5];
            static const int W[5] = {4, 4, 4, 8, 8};
            size_t pos = 0;
            for (int k = 0; k < 5; k++) {
                if (!read_field(ln, pos, (size_t)W[k], k < 3 ? 0 : 2, k < 3, v[k])) return DGPU_ERR_ARG;
                pos += (size_t)W[k];
            }
            for (int k = 0; k < 3; k++) hkl.push_back((int32_t)v[k]);
            iobs.push_back(v[3]);
        }
    } else {
        size_t k = 0;
        while (k < lines.size() && lines[k].compare(0, 14, "_refln_index_h") != 0) k++;
        if (k == lines.size()) return DGPU_ERR_ARG;
        int j_h = 0, j_k = 0, j_l = 0, j = 1;
        for (; k < lines.size(); k++) {
            const std::string &ln = lines[k];
            if ((!ln.empty() && ln[0] == '#') || rtrim(ln).empty()) continue;
            if (ln.compare(0, 14, "_refln_index_h") == 0) j_h = j;
            if (ln.compare(0, 14, "_refln_index_k") == 0) j_k = j;
            if (ln.compare(0, 14, "_refln_index_l") == 0) j_l = j;
            if (ln.compare(0, 21, "_refln_F_squared_calc") == 0) j_icalc = j;
            if (ln.compare(0, 7, "_refln_") != 0) break;
            nentries++;
            j++;
        }
        if (j_h != 1 || j_k != 2 || j_l != 3 || nentries < 4 || nentries - 1 - 3 > 3) return DGPU_ERR_ARG;
        for (; k < lines.size(); k++) {
            const auto t = blank_tokens(lines[k]);
            if (t.empty()) continue;
            if (t.size() < nentries - 1) return DGPU_ERR_ARG;
            std::vector<double> r(nentries - 1);
            for (size_t q = 0; q + 1 < nentries; q++) {
                char *end = nullptr;
                r[q] = strtod(t[q].c_str(), &end);
                if (*end) return DGPU_ERR_ARG;
            }
            for (int a = 0; a < 3; a++) hkl.push_back((int32_t)lround(r[(size_t)a]));
            rows.push_back(r);
        }
    }
    const int64_t n = (int64_t)hkl.size() / 3;
    std::vector<double> ic((size_t)n), sg((size_t)n), ph((size_t)n);
    if (n > 0) {
        const int rc = dgpu_calc_hkl(ctx, cr, opts, hkl.data(), n, scale, exti, rlambda, ic.data(), sg.data(),
                                     ph.data());
        if (rc != DGPU_OK) return rc;
    }
    // calcfile and the list file (.fcf) (fourier_sup.f90:3289-3303, 3487-3548)
    const std::string cf(calcfile);
    std::string lf = cf;
    if (lf.size() >= 3 && lf.compare(lf.size() - 3, 3, "hkl") == 0) lf.replace(lf.size() - 3, 3, "fcf");
    else lf += ".fcf";
    Sink w(cf), ls(lf);
    if (!w.f || !ls.f) return DGPU_ERR_IO;
    for (int64_t r = 0; r < n; r++) {
        const int h = hkl[3 * r], k = hkl[3 * r + 1], l = hkl[3 * r + 2];
        const std::string ihkl = edit_i(4, h) + edit_i(4, k) + edit_i(4, l);
        if (h == 0 && k == 0 && l == 0) {
            w.rec(ihkl + edit_f(8, 2, 0.0) + edit_f(8, 2, 0.0));
            continue;
        }
        const double qq = ic[(size_t)r];
        if (style == DGPU_HKL_HKLF4) {
            w.rec(ihkl + edit_f(8, 2, qq) + edit_f(8, 2, sg[(size_t)r]));
            ls.rec(ihkl + edit_f(10, 2, sqrt(fabs(iobs[(size_t)r]))) + edit_f(10, 2, sqrt(fabs(qq))) +
                   edit_f(7, 2, ph[(size_t)r]));
        } else {
            std::vector<double> vals = rows[(size_t)r];
            if (j_icalc != 0 && (size_t)j_icalc <= vals.size()) vals[(size_t)j_icalc - 1] = qq;
            std::string s = ihkl;
            for (size_t q = 3; q < vals.size(); q++) s += edit_f(12, 2, vals[q]);
            w.rec(s);
            ls.rec(ihkl + edit_f(10, 2, vals[0]) + edit_f(10, 2, sqrt(fabs(qq))) + edit_f(7, 2, ph[(size_t)r]));
        }
    }
    const bool ok1 = w.close(), ok2 = ls.close();
    return ok1 && ok2 ? DGPU_OK : DGPU_ERR_IO;
}

}  // extern "C"
