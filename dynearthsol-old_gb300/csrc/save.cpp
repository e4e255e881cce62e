// The .save file of one output frame, as Output::_write (output.cxx:73-198)
// writes it through BinaryOutput (binaryio.cxx:44-131), from host arrays in
// the reference's layout, and the .chkpt file (output.cxx:270-296), each with
// the marker sets it is given.  Derived element fields (density, mesh
// quality, viscosity, material) and marker coordinates are computed here on
// the host with the reference's arithmetic and libm, so the files match the
// reference's byte for byte.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "des_gpu.h"

namespace {

constexpr std::size_t kHeaderLen = 4096;
const char kRevision[] = "# DynEarthSol ndims=3 revision=3\n";

// binaryio.cxx: a 4096-byte text header of "name\tposition\n" lines, the
// arrays after it
class SaveFile {
public:
    explicit SaveFile(const char *path) : f_(std::fopen(path, "wb")), header_(kHeaderLen, '\0')
    {
        std::memcpy(header_.data(), kRevision, sizeof(kRevision) - 1);
        used_ = sizeof(kRevision) - 1;
        if (f_) std::fseek(f_, (long)kHeaderLen, SEEK_SET);
    }
    ~SaveFile() { close(); }
    bool ok() const { return f_ != nullptr && !failed_; }
    template <class T>
    void write(const T *a, std::size_t count, const char *name)
    {
        if (!f_) return;
        char line[256];
        int len = std::snprintf(line, sizeof line, "%s\t%ld\n", name, (long)eof_);
        if (len <= 0 || len >= (int)sizeof line || used_ + (std::size_t)len >= kHeaderLen) {
            failed_ = true;
            return;
        }
        std::memcpy(header_.data() + used_, line, (std::size_t)len);
        used_ += (std::size_t)len;
        std::size_t n = std::fwrite(a, sizeof(T), count, f_);
        if (n != count) failed_ = true;
        eof_ += n * sizeof(T);
    }
    int close()
    {
        if (!f_) return failed_ ? DES_ERR_ARG : DES_OK;
        std::fseek(f_, 0, SEEK_SET);
        if (std::fwrite(header_.data(), 1, kHeaderLen, f_) != kHeaderLen) failed_ = true;
        if (std::fclose(f_) != 0) failed_ = true;
        f_ = nullptr;
        return failed_ ? DES_ERR_ARG : DES_OK;
    }

private:
    std::FILE *f_;
    std::vector<char> header_;
    std::size_t used_ = 0, eof_ = kHeaderLen;
    bool failed_ = false;
};

double mv(const des_matvec &v, int m) { return v.len == 1 ? v.v[0] : v.v[m]; }

double elem_T(const int *conn, const double *T, int e)
{
    double t = 0;
    for (int i = 0; i < 4; ++i) t += T[conn[4 * (std::size_t)e + i]];
    t /= 4;
    return t;
}

// geometry.cxx:53-83 (3D)
double triangle_area(const double *a, const double *b, const double *c)
{
    double ab0 = b[0] - a[0], ab1 = b[1] - a[1];
    double ac0 = c[0] - a[0], ac1 = c[1] - a[1];
    double ab2 = b[2] - a[2], ac2 = c[2] - a[2];
    double d0 = ab1 * ac2 - ab2 * ac1;
    double d1 = ab2 * ac0 - ab0 * ac2;
    double d2 = ab0 * ac1 - ab1 * ac0;
    return std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) / 2;
}

// geometry.cxx:472-509 (3D)
double elem_quality(const double *coord, const int *conn, const double *volume, int e)
{
    const int *c = conn + 4 * (std::size_t)e;
    const double *a = coord + 3 * (std::size_t)c[0], *b = coord + 3 * (std::size_t)c[1];
    const double *cc = coord + 3 * (std::size_t)c[2], *d = coord + 3 * (std::size_t)c[3];
    double vol = volume[e];
    double normalization_factor = 216 * std::sqrt(3);
    double area_sum = (triangle_area(a, b, cc) + triangle_area(a, b, d) + triangle_area(cc, d, a) +
                       triangle_area(cc, d, b));
    return normalization_factor * vol * vol / (area_sum * area_sum * area_sum);
}

// matprops.cxx:707-728
double rho(const des_params &p, const int *markers, int nmat, const int *conn, const double *T, int e)
{
    const double celsius0 = 273;
    double TinCelsius = elem_T(conn, T, e) - celsius0;
    double result = 0;
    int n = 0;
    const int *k = markers + (std::size_t)nmat * e;
    for (int m = 0; m < nmat; m++) {
        result += mv(p.rho0, m) * (1 - mv(p.alpha, m) * TinCelsius) * k[m];
        n += k[m];
    }
    return result / n;
}

// utils.hpp:78-87
double second_invariant(const double *t)
{
    double a = (t[0] + t[1] + t[2]) / 3;
    return std::sqrt(0.5 * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a)) +
                     t[3] * t[3] + t[4] * t[4] + t[5] * t[5]);
}

// matprops.cxx:607-643
double visc(const des_params &p, const int *markers, int nmat, const int *conn, const double *T,
            const double *srate, int e)
{
    const double gas_constant = 8.3144;
    const double min_strain_rate = 1e-30;
    double t = elem_T(conn, T, e);
    double edot = second_invariant(srate + 6 * (std::size_t)e);
    edot = std::max(edot, min_strain_rate);
    double result = 0;
    int n = 0;
    const int *k = markers + (std::size_t)nmat * e;
    for (int m = 0; m < nmat; m++) {
        double ve = mv(p.visc_exponent, m);
        double pw = 1 / ve - 1;
        double pw1 = -1 / ve;
        double visc0 = 0.25 * std::pow(edot, pw) * std::pow(0.75 * mv(p.visc_coefficient, m), pw1) *
                       std::exp(mv(p.visc_activation_energy, m) / (ve * gas_constant * t)) * 1e6;
        result += k[m] / visc0;
        n += k[m];
    }
    double v = n / result;
    return std::min(std::max(v, p.visc_min), p.visc_max);
}

// checks one marker set against the mesh it refers to
int check_set(const des_marker_set &ms, int nelem)
{
    if (!ms.name || ms.nmarkers < 0) return DES_ERR_ARG;
    if (ms.nmarkers > 0 && (!ms.eta || !ms.elem || !ms.mattype || !ms.id)) return DES_ERR_ARG;
    for (int i = 0; i < ms.nmarkers; ++i)
        if (ms.elem[i] < 0 || ms.elem[i] >= nelem) return DES_ERR_ARG;
    return DES_OK;
}

int check_sets(const des_marker_set *sets, int nsets, int nelem)
{
    if (nsets < 0 || (nsets > 0 && !sets)) return DES_ERR_ARG;
    for (int k = 0; k < nsets; ++k)
        if (int rc = check_set(sets[k], nelem)) return rc;
    return DES_OK;
}

std::string field(const des_marker_set &ms, const char *suffix) { return std::string(ms.name) + suffix; }

// MarkerSet::write_save_file (markerset.cxx:452-483): the markers' positions
// x_j = sum_k eta_k x(conn_k)_j, in that order from zero
void write_set_save(SaveFile &bin, const des_marker_set &ms, const int *conn, const double *coord)
{
    const int n = ms.nmarkers;
    bin.write(&n, 1, field(ms, " size").c_str());
    std::vector<double> mc(3 * (std::size_t)n, 0.0);
    for (int i = 0; i < n; ++i) {
        const int *c = conn + 4 * (std::size_t)ms.elem[i];
        const double *eta = ms.eta + 4 * (std::size_t)i;
        double *x = mc.data() + 3 * (std::size_t)i;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 4; k++) x[j] += eta[k] * coord[3 * (std::size_t)c[k] + j];
    }
    bin.write(mc.data(), 3 * (std::size_t)n, field(ms, ".coord").c_str());
    bin.write(ms.elem, (std::size_t)n, field(ms, ".elem").c_str());
    bin.write(ms.mattype, (std::size_t)n, field(ms, ".mattype").c_str());
    bin.write(ms.id, (std::size_t)n, field(ms, ".id").c_str());
}

// MarkerSet::write_chkpt_file (markerset.cxx:407-419)
void write_set_chkpt(SaveFile &bin, const des_marker_set &ms)
{
    const int n = ms.nmarkers;
    const int size[2] = {n, ms.last_id};
    bin.write(size, 2, field(ms, " size").c_str());
    bin.write(ms.eta, 4 * (std::size_t)n, field(ms, ".eta").c_str());
    bin.write(ms.elem, (std::size_t)n, field(ms, ".elem").c_str());
    bin.write(ms.mattype, (std::size_t)n, field(ms, ".mattype").c_str());
    bin.write(ms.id, (std::size_t)n, field(ms, ".id").c_str());
}

}  // namespace

extern "C" int des_write_save(const char *path, const des_mesh_view *m, const des_params *p,
                              const unsigned *bcflag, const des_state_view *s, const des_save_averages *avg,
                              const des_marker_set *sets, int nsets)
{
    if (!path || !m || !p || !bcflag || !s || !m->connectivity || !m->elemmarkers) return DES_ERR_ARG;
    if (s->nnode != m->nnode || s->nelem != m->nelem) return DES_ERR_ARG;
    if (!s->coord || !s->vel || !s->temperature || !s->plstrain || !s->delta_plstrain || !s->strain_rate ||
        !s->strain || !s->stress || !s->volume || !s->force || !s->coord0)
        return DES_ERR_ARG;
    if (avg && (!avg->coord0 || !avg->strain0 || !avg->stress_sum || !avg->dpls_sum || avg->interval < 1))
        return DES_ERR_ARG;
    if (check_sets(sets, nsets, m->nelem)) return DES_ERR_ARG;
    const std::size_t N = m->nnode, E = m->nelem;
    const int *conn = m->connectivity;
    SaveFile bin(path);
    if (!bin.ok()) return DES_ERR_ARG;
    double inv_dt = 0;
    if (avg) inv_dt = 1.0 / (s->time - avg->time0);
    bin.write(s->coord, 3 * N, "coordinate");
    bin.write(conn, 4 * E, "connectivity");
    bin.write(s->vel, 3 * N, "velocity");
    if (avg) {
        std::vector<double> c0(avg->coord0, avg->coord0 + 3 * N);
        for (std::size_t i = 0; i < 3 * N; ++i) c0[i] = (s->coord[i] - c0[i]) * inv_dt;
        bin.write(c0.data(), 3 * N, "velocity averaged");
    }
    bin.write(s->temperature, N, "temperature");
    bin.write(s->plstrain, E, "plastic strain");
    if (avg) {
        std::vector<double> d(avg->dpls_sum, avg->dpls_sum + E);
        for (std::size_t i = 0; i < E; ++i) d[i] *= inv_dt;
        bin.write(d.data(), E, "plastic strain-rate");
        std::vector<double> s0(avg->strain0, avg->strain0 + 6 * E);
        for (std::size_t i = 0; i < 6 * E; ++i) s0[i] = (s->strain[i] - s0[i]) * inv_dt;
        bin.write(s0.data(), 6 * E, "strain-rate");
    } else {
        bin.write(s->delta_plstrain, E, "plastic strain-rate");
        bin.write(s->strain_rate, 6 * E, "strain-rate");
    }
    bin.write(s->strain, 6 * E, "strain");
    bin.write(s->stress, 6 * E, "stress");
    if (avg) {
        std::vector<double> sa(avg->stress_sum, avg->stress_sum + 6 * E);
        double tmp = 1.0 / (avg->interval + 1);
        for (std::size_t i = 0; i < 6 * E; ++i) sa[i] *= tmp;
        bin.write(sa.data(), 6 * E, "stress averaged");
    }
    std::vector<double> tmp(E);
    for (std::size_t e = 0; e < E; ++e) tmp[e] = rho(*p, m->elemmarkers, m->nmat, conn, s->temperature, (int)e);
    bin.write(tmp.data(), E, "density");
    for (std::size_t e = 0; e < E; ++e) tmp[e] = elem_quality(s->coord, conn, s->volume, (int)e);
    bin.write(tmp.data(), E, "mesh quality");
    for (std::size_t e = 0; e < E; ++e)
        tmp[e] = visc(*p, m->elemmarkers, m->nmat, conn, s->temperature, s->strain_rate, (int)e);
    bin.write(tmp.data(), E, "viscosity");
    for (std::size_t e = 0; e < E; ++e) {
        // the most abundant material of the element (the first on a tie)
        const int *k = m->elemmarkers + (std::size_t)m->nmat * e;
        tmp[e] = (double)(std::max_element(k, k + m->nmat) - k);
    }
    bin.write(tmp.data(), E, "material");
    bin.write(s->force, 3 * N, "force");
    bin.write(s->coord0, 3 * N, "coord0");
    bin.write(bcflag, N, "bcflag");
    for (int k = 0; k < nsets; ++k) write_set_save(bin, sets[k], conn, s->coord);
    return bin.close();
}

// Output::write_checkpoint (output.cxx:270-296) in 3D: time and
// compensation pressure, segments, segment flags, volume_old, then the
// marker sets.
extern "C" int des_write_checkpoint(const char *path, const des_mesh_view *m, double time,
                                    double compensation_pressure, const double *volume_old,
                                    const des_marker_set *sets, int nsets)
{
    if (!path || !m || !volume_old || (m->nseg > 0 && (!m->segment || !m->segflag))) return DES_ERR_ARG;
    if (check_sets(sets, nsets, m->nelem)) return DES_ERR_ARG;
    SaveFile bin(path);
    if (!bin.ok()) return DES_ERR_ARG;
    const double tc[2] = {time, compensation_pressure};
    bin.write(tc, 2, "time compensation_pressure");
    bin.write(m->segment, 3 * (std::size_t)m->nseg, "segment");
    bin.write(m->segflag, (std::size_t)m->nseg, "segflag");
    bin.write(volume_old, (std::size_t)m->nelem, "volume_old");
    for (int k = 0; k < nsets; ++k) write_set_chkpt(bin, sets[k]);
    return bin.close();
}
