// Minimal, headless stand-ins for the handful of Qt / QGLViewer types that the
// reference's CPU solver files (TetMesh, IsotropicMaterial,
// IsotropicNeohookeanMaterial, DescentOptimize) name in their headers.
//
// This is test infrastructure: it lets the reference CPU path compile
// unmodified with g++ so that it can act as the parity oracle.  Nothing here
// renders anything; the drawing entry points of TetMesh are never called.
//
// QFile path handling: the reference opens its mesh through hard-coded
// Windows-style relative paths ("..\\model\\armadillo\\armadillo.1.node",
// TetMesh.cpp:179-181).  Backslashes are mapped to '/', and when
// phybs_shim_set_mesh_stem() has been given a stem, any path that ends in
// "armadillo.1.<ext>" is redirected to "<stem>.<ext>".  That is how the
// harness injects synthetic meshes.
#pragma once

#include <string>
#include <vector>
#include <fstream>
#include <sstream>
#include <iostream>
#include <cstdio>
#include <cstdlib>

void phybs_shim_set_mesh_stem(const std::string &stem);
const std::string &phybs_shim_mesh_stem();

class QString {
public:
    QString() {}
    QString(const char *s) : s_(s ? s : "") {}
    QString(const std::string &s) : s_(s) {}
    QString simplified() const {
        std::string out;
        bool pending_space = false;
        for (char c : s_) {
            bool ws = (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f');
            if (ws) { pending_space = !out.empty(); continue; }
            if (pending_space) out.push_back(' ');
            pending_space = false;
            out.push_back(c);
        }
        return QString(out);
    }
    std::vector<QString> split(const QString &sep) const {
        std::vector<QString> parts;
        const std::string &d = sep.s_;
        size_t start = 0;
        if (d.empty()) { parts.push_back(*this); return parts; }
        for (;;) {
            size_t p = s_.find(d, start);
            if (p == std::string::npos) { parts.push_back(QString(s_.substr(start))); break; }
            parts.push_back(QString(s_.substr(start, p - start)));
            start = p + d.size();
        }
        return parts;
    }
    int toInt() const { return std::atoi(s_.c_str()); }
    const std::string &str() const { return s_; }
private:
    std::string s_;
};
typedef std::vector<QString> QStringList;
#define QStringLiteral(x) QString(x)

struct QIODevice {
    enum OpenModeFlag { NotOpen = 0, ReadOnly = 1, WriteOnly = 2, ReadWrite = 3, Append = 4, Truncate = 8, Text = 16 };
};

class QFile {
public:
    explicit QFile(const QString &name) : name_(map_path(name.str())) {}
    bool open(int mode) {
        std::ios::openmode m = std::ios::in;
        if ((mode & QIODevice::ReadWrite) == QIODevice::ReadWrite) m = std::ios::in | std::ios::out | std::ios::trunc;
        else if (mode & QIODevice::WriteOnly) m = std::ios::out | std::ios::trunc;
        fs_.open(name_, m);
        return fs_.is_open();
    }
    void close() { if (fs_.is_open()) fs_.close(); }
    std::fstream &stream() { return fs_; }
private:
    static std::string map_path(std::string p) {
        for (auto &c : p) if (c == '\\') c = '/';
        const std::string &stem = phybs_shim_mesh_stem();
        const std::string key = "armadillo.1.";
        size_t k = p.rfind(key);
        if (!stem.empty() && k != std::string::npos)
            return stem + "." + p.substr(k + key.size());
        return p;
    }
    std::string name_;
    std::fstream fs_;
};

class QTextStream {
public:
    explicit QTextStream(QFile *f) : fs_(&f->stream()) {}
    bool atEnd() { return fs_->peek() == std::char_traits<char>::eof(); }
    QString readLine() { std::string l; std::getline(*fs_, l); return QString(l); }
    template <typename T> QTextStream &operator>>(T &v) { (*fs_) >> v; return *this; }
    QTextStream &operator<<(const char *s) { (*fs_) << s; return *this; }
    QTextStream &operator<<(const QString &s) { (*fs_) << s.str(); return *this; }
    template <typename T> QTextStream &operator<<(const T &v) { (*fs_) << v; return *this; }
    QTextStream &operator<<(QTextStream &(*manip)(QTextStream &)) { return manip(*this); }
    std::fstream &raw() { return *fs_; }
private:
    std::fstream *fs_;
};
inline QTextStream &endl(QTextStream &s) { s.raw() << '\n'; s.raw().flush(); return s; }

class QTime {
public:
    void start() {}
    int restart() { return 0; }
    int elapsed() const { return 0; }
};
class QElapsedTimer {
public:
    void start() {}
    int restart() { return 0; }
    long long elapsed() const { return 0; }
    void invalidate() {}
};

// Types named only by RenderWidget.h's class declaration (never instantiated).
class QWidget {};
class QPainter {};
class QPaintEvent {};
class QMouseEvent {};
class QKeyEvent {};
class QGLViewer {
public:
    explicit QGLViewer(QWidget * = nullptr) {}
    virtual ~QGLViewer() {}
};

typedef double GLdouble;
typedef int GLint;
typedef float GLfloat;
typedef unsigned int GLenum;
#ifndef GL_FALSE
#define GL_FALSE 0
#define GL_TRUE 1
#define GL_TRIANGLES 0x0004
#define GL_POINTS 0x0000
#endif
// TetMesh::drawTetBoundFace / drawDraggedNodes reference these; they are never
// called by the oracle and do nothing.
inline void glColor3f(GLfloat, GLfloat, GLfloat) {}
inline void glBegin(GLenum) {}
inline void glEnd() {}
inline void glNormal3fv(const GLfloat *) {}
inline void glVertex3fv(const GLfloat *) {}
inline void glPointSize(GLfloat) {}
