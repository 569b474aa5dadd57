// qtshim.h -- the few Qt classes the reference's CPU engines, trees, data
// model and solvers use, restated on the C++ standard library so that those
// sources compile unchanged without Qt.  TEST INFRASTRUCTURE ONLY: it exists to
// build the reference's own code into oracle/_ref (the checker of the oracle
// restatement); nothing in the GB300 engine includes it.
//
// Covered: QDebug / qDebug (messages discarded unless NBODY_REF_DEBUG is set in
// the environment), QChar, QString (arg, compare, indexOf, mid, trimmed,
// split, toDouble, toULongLong, contains, isEmpty), QStringList, QFile and
// QTextStream (text read/write of nbody_data::load/save), QVariant and
// QVariantMap (the factories' parameter maps), QVector, QPair, Q_UNUSED,
// Q_ASSERT, QT_VERSION, and the GLint / GLenum / GL_FLOAT / GL_DOUBLE type
// tokens that nbtype_info.h names.
#pragma once

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include <sys/stat.h>

#define QT_VERSION_CHECK(major, minor, patch) (((major) << 16) | ((minor) << 8) | (patch))
#define QT_VERSION QT_VERSION_CHECK(5, 15, 0)
#define Q_UNUSED(x) (void)(x)
#define Q_ASSERT(x) ((void)0)

typedef int GLint;
typedef unsigned int GLenum;
#ifndef GL_FLOAT
#define GL_FLOAT 0x1406
#endif
#ifndef GL_DOUBLE
#define GL_DOUBLE 0x140A
#endif

namespace Qt {
enum CaseSensitivity { CaseInsensitive, CaseSensitive };
enum Initialization { Uninitialized };
}  // namespace Qt

class QChar {
public:
    QChar(char c = ' ') : c_(c) {}
    char toLatin1() const { return c_; }
private:
    char c_;
};

class QString;
typedef std::vector<QString> QStringList_base;

class QString {
public:
    enum SplitBehavior { KeepEmptyParts, SkipEmptyParts };
    QString() {}
    QString(const char* s) : s_(s ? s : "") {}
    QString(const std::string& s) : s_(s) {}
    QString(QChar c) : s_(1, c.toLatin1()) {}
    const std::string& str() const { return s_; }
    std::string toStdString() const { return s_; }
    bool isEmpty() const { return s_.empty(); }
    int size() const { return (int)s_.size(); }
    int length() const { return (int)s_.size(); }
    bool operator==(const QString& o) const { return s_ == o.s_; }
    bool operator==(const char* o) const { return s_ == o; }
    bool operator!=(const QString& o) const { return s_ != o.s_; }
    bool operator<(const QString& o) const { return s_ < o.s_; }
    QString operator+(const QString& o) const { return QString(s_ + o.s_); }
    QString& operator+=(const QString& o) { s_ += o.s_; return *this; }
    bool contains(const QString& o) const { return s_.find(o.s_) != std::string::npos; }
    bool startsWith(const QString& o) const { return s_.compare(0, o.s_.size(), o.s_) == 0; }
    bool endsWith(const QString& o) const {
        return s_.size() >= o.s_.size() && s_.compare(s_.size() - o.s_.size(), o.s_.size(), o.s_) == 0;
    }
    int indexOf(const QString& o, int from = 0) const {
        const size_t p = s_.find(o.s_, (size_t)from);
        return p == std::string::npos ? -1 : (int)p;
    }
    QString mid(int pos, int n = -1) const {
        if (pos < 0 || pos > (int)s_.size()) return QString();
        return QString(n < 0 ? s_.substr(pos) : s_.substr(pos, n));
    }
    QString trimmed() const {
        size_t a = 0, b = s_.size();
        while (a < b && std::isspace((unsigned char)s_[a])) ++a;
        while (b > a && std::isspace((unsigned char)s_[b - 1])) --b;
        return QString(s_.substr(a, b - a));
    }
    QString repeated(int k) const {
        std::string r;
        for (int i = 0; i < k; ++i) r += s_;
        return QString(r);
    }
    static std::string lower(const std::string& x) {
        std::string r(x);
        for (char& c : r) c = (char)std::tolower((unsigned char)c);
        return r;
    }
    int compare(const QString& o, Qt::CaseSensitivity cs = Qt::CaseSensitive) const {
        const std::string a = cs == Qt::CaseSensitive ? s_ : lower(s_);
        const std::string b = cs == Qt::CaseSensitive ? o.s_ : lower(o.s_);
        return a.compare(b);
    }
    std::vector<QString> split(const QString& sep, SplitBehavior sb = KeepEmptyParts) const {
        std::vector<QString> out;
        size_t start = 0;
        while (true) {
            const size_t p = sep.s_.empty() ? std::string::npos : s_.find(sep.s_, start);
            const std::string part = s_.substr(start, p == std::string::npos ? std::string::npos
                                                                              : p - start);
            if (!(sb == SkipEmptyParts && part.empty())) out.push_back(QString(part));
            if (p == std::string::npos) break;
            start = p + sep.s_.size();
        }
        return out;
    }
    std::vector<QString> split(QChar sep, SplitBehavior sb = KeepEmptyParts) const {
        return split(QString(sep), sb);
    }
    double toDouble(bool* ok = nullptr) const {
        const std::string t = trimmed().s_;
        char* end = nullptr;
        const double v = std::strtod(t.c_str(), &end);
        const bool good = !t.empty() && end != nullptr && *end == '\0';
        if (ok) *ok = good;
        return good ? v : 0.0;
    }
    unsigned long long toULongLong(bool* ok = nullptr, int base = 10) const {
        const std::string t = trimmed().s_;
        char* end = nullptr;
        const unsigned long long v = std::strtoull(t.c_str(), &end, base);
        const bool good = !t.empty() && t[0] != '-' && end != nullptr && *end == '\0';
        if (ok) *ok = good;
        return good ? v : 0ull;
    }
    int toInt(bool* ok = nullptr, int base = 10) const {
        const std::string t = trimmed().s_;
        char* end = nullptr;
        const long v = std::strtol(t.c_str(), &end, base);
        const bool good = !t.empty() && end != nullptr && *end == '\0';
        if (ok) *ok = good;
        return good ? (int)v : 0;
    }
    // "%1"-style argument substitution (the lowest-numbered marker)
    QString arg(const QString& a) const { return subst(a.s_); }
    QString arg(const char* a) const { return subst(a); }
    template <class I, class = typename std::enable_if<std::is_integral<I>::value>::type>
    QString arg(I v, int width = 0, int base = 10, QChar fill = QChar(' ')) const {
        char buf[96];
        if (base == 16)
            std::snprintf(buf, sizeof(buf), "%llx", (unsigned long long)v);
        else if (std::is_signed<I>::value)
            std::snprintf(buf, sizeof(buf), "%lld", (long long)v);
        else
            std::snprintf(buf, sizeof(buf), "%llu", (unsigned long long)v);
        return subst(pad(buf, width, fill));
    }
    QString arg(double v, int width = 0, char fmt = 'g', int prec = -1,
                QChar fill = QChar(' ')) const {
        char spec[16], buf[128];
        std::snprintf(spec, sizeof(spec), "%%.%d%c", prec < 0 ? 6 : prec, fmt);
        std::snprintf(buf, sizeof(buf), spec, v);
        return subst(pad(buf, width, fill));
    }
    static QString number(double v) {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%g", v);
        return QString(buf);
    }
    template <class I>
    static typename std::enable_if<std::is_integral<I>::value, QString>::type number(I v) {
        return QString(std::is_signed<I>::value ? std::to_string((long long)v)
                                                : std::to_string((unsigned long long)v));
    }
    void clear() { s_.clear(); }
    long long toLongLong(bool* ok = nullptr, int base = 10) const {
        const std::string t = trimmed().s_;
        char* end = nullptr;
        const long long v = std::strtoll(t.c_str(), &end, base);
        const bool good = !t.empty() && end != nullptr && *end == '\0';
        if (ok) *ok = good;
        return good ? v : 0ll;
    }

private:
    static std::string pad(const std::string& x, int width, QChar fill) {
        if ((int)x.size() >= width) return x;
        return std::string(width - x.size(), fill.toLatin1()) + x;
    }
    QString subst(const std::string& a) const {
        int best = 100;
        size_t at = std::string::npos, len = 0;
        for (size_t i = 0; i + 1 < s_.size(); ++i) {
            if (s_[i] != '%' || !std::isdigit((unsigned char)s_[i + 1])) continue;
            const int k = s_[i + 1] - '0';
            if (k < best) {
                best = k;
                at = i;
                len = 2;
            }
        }
        if (at == std::string::npos) return *this;
        return QString(s_.substr(0, at) + a + s_.substr(at + len));
    }
    std::string s_;
};

class QStringList : public std::vector<QString> {
public:
    QStringList() {}
    QStringList(const std::vector<QString>& v) : std::vector<QString>(v) {}
};

template <class T>
class QVector : public std::vector<T> {
public:
    void resize(int n) { std::vector<T>::resize((size_t)n); }
};

template <class A, class B>
using QPair = std::pair<A, B>;

class QVariant {
public:
    QVariant() {}
    QVariant(const char* s) : s_(s) {}
    QVariant(const QString& s) : s_(s.str()) {}
    QVariant(double v) { char b[64]; std::snprintf(b, sizeof(b), "%.17g", v); s_ = b; }
    QVariant(int v) : s_(std::to_string(v)) {}
    QVariant(long long v) : s_(std::to_string(v)) {}
    QVariant(unsigned long long v) : s_(std::to_string(v)) {}
    QVariant(bool v) : s_(v ? "true" : "false") {}
    QString toString() const { return QString(s_); }
    double toDouble(bool* ok = nullptr) const { return QString(s_).toDouble(ok); }
    unsigned long long toULongLong(bool* ok = nullptr) const { return QString(s_).toULongLong(ok); }
    unsigned int toUInt(bool* ok = nullptr) const { return (unsigned)QString(s_).toULongLong(ok); }
    int toInt(bool* ok = nullptr) const { return QString(s_).toInt(ok); }
    bool toBool() const { return s_ == "true" || s_ == "1"; }
    bool isValid() const { return !s_.empty(); }
private:
    std::string s_;
};

class QVariantMap : public std::map<QString, QVariant> {
public:
    QVariant value(const QString& k, const QVariant& dflt = QVariant()) const {
        auto it = find(k);
        return it == end() ? dflt : it->second;
    }
    bool contains(const QString& k) const { return find(k) != end(); }
};

class QDebug {
public:
    QDebug() : on_(std::getenv("NBODY_REF_DEBUG") != nullptr) {}
    QDebug(const QDebug& o) : on_(o.on_) {}
    ~QDebug() {
        if (on_ && !buf_.empty()) std::fprintf(stderr, "%s\n", buf_.c_str());
    }
    QDebug& noquote() { return *this; }
    QDebug& operator<<(const char* s) { return put(s ? s : ""); }
    QDebug& operator<<(const std::string& s) { return put(s); }
    QDebug& operator<<(const QString& s) { return put(s.str()); }
    QDebug& operator<<(char c) { return put(std::string(1, c)); }
    QDebug& operator<<(bool b) { return put(b ? "true" : "false"); }
    QDebug& operator<<(const void* p) { char b[32]; std::snprintf(b, sizeof(b), "%p", p); return put(b); }
    template <class T>
    typename std::enable_if<std::is_arithmetic<T>::value, QDebug&>::type operator<<(T v) {
        char b[64];
        if (std::is_floating_point<T>::value) std::snprintf(b, sizeof(b), "%g", (double)v);
        else if (std::is_signed<T>::value) std::snprintf(b, sizeof(b), "%lld", (long long)v);
        else std::snprintf(b, sizeof(b), "%llu", (unsigned long long)v);
        return put(b);
    }
    template <class T>
    typename std::enable_if<std::is_enum<T>::value, QDebug&>::type operator<<(T v) {
        return *this << (long long)v;
    }
    template <class T>
    QDebug& operator<<(const std::vector<T>& v) {
        put("(");
        for (const T& x : v) *this << x;
        return put(")");
    }
private:
    QDebug& put(const std::string& s) {
        if (on_) {
            if (!buf_.empty()) buf_ += ' ';
            buf_ += s;
        }
        return *this;
    }
    bool on_;
    std::string buf_;
};

inline QDebug qDebug() { return QDebug(); }
inline QDebug qWarning() { return QDebug(); }

typedef long long qint64;
typedef unsigned long long quint64;

class QFile {
public:
    enum OpenModeFlag { NotOpen = 0, ReadOnly = 1, WriteOnly = 2, ReadWrite = 3, Append = 4,
                        Truncate = 8, Text = 16 };
    typedef int OpenMode;
    QFile() {}
    explicit QFile(const QString& name) : name_(name.str()) {}
    ~QFile() { close(); }
    void setFileName(const QString& name) { name_ = name.str(); }
    QString fileName() const { return QString(name_); }
    bool open(OpenMode mode) {
        close();
        const char* m = (mode & Append) ? "ab" : (mode & WriteOnly) ? "wb" : "rb";
        f_ = std::fopen(name_.c_str(), m);
        err_ = f_ ? 0 : errno;
        return f_ != nullptr;
    }
    bool isOpen() const { return f_ != nullptr; }
    void close() {
        if (f_) std::fclose(f_);
        f_ = nullptr;
    }
    bool flush() { return f_ && std::fflush(f_) == 0; }
    qint64 write(const char* data, qint64 len) {
        return f_ ? (qint64)std::fwrite(data, 1, (size_t)len, f_) : -1;
    }
    qint64 read(char* data, qint64 len) {
        return f_ ? (qint64)std::fread(data, 1, (size_t)len, f_) : -1;
    }
    qint64 pos() const { return f_ ? (qint64)std::ftell(f_) : 0; }
    bool seek(qint64 p) { return f_ && std::fseek(f_, (long)p, SEEK_SET) == 0; }
    qint64 size() const {
        std::FILE* g = std::fopen(name_.c_str(), "rb");
        if (!g) return 0;
        std::fseek(g, 0, SEEK_END);
        const long n = std::ftell(g);
        std::fclose(g);
        return n;
    }
    QString errorString() const { return QString(std::strerror(err_ ? err_ : errno)); }
    std::FILE* handle() { return f_; }
private:
    std::string name_;
    std::FILE* f_ = nullptr;
    int err_ = 0;
};

class QDir {
public:
    explicit QDir(const std::string& path) : path_(path) {}
    // creates the directory and its parents (mkdir -p of path / sub)
    bool mkpath(const QString& sub) const {
        std::string full = path_.empty() ? sub.str() : path_ + "/" + sub.str();
        std::string cur;
        for (size_t i = 0; i <= full.size(); ++i) {
            if (i == full.size() || full[i] == '/') {
                if (!cur.empty()) mkdir_one(cur);
            }
            if (i < full.size()) cur += full[i];
        }
        return true;
    }
private:
    static void mkdir_one(const std::string& d);
    std::string path_;
};

class QFileInfo {
public:
    explicit QFileInfo(const QString& name) : name_(name.str()) {}
    QDir dir() const {
        const size_t p = name_.rfind('/');
        return QDir(p == std::string::npos ? std::string(".") : name_.substr(0, p));
    }
private:
    std::string name_;
};

class QTextStream {
public:
    enum RealNumberNotation { SmartNotation, FixedNotation, ScientificNotation };
    enum NumberFlag { ShowBase = 1, ForcePoint = 2, ForceSign = 4, UppercaseBase = 8,
                      UppercaseDigits = 16 };
    QTextStream() {}
    explicit QTextStream(QFile* f) : file_(f) {}
    void setDevice(QFile* f) { file_ = f; }
    void setRealNumberPrecision(int p) { prec_ = p; }
    void setRealNumberNotation(RealNumberNotation n) { nota_ = n; }
    void setNumberFlags(int fl) { flags_ = fl; }
    void flush() { if (fp()) std::fflush(fp()); }
    bool atEnd() {
        if (fp() == nullptr) return true;
        const int c = std::fgetc(fp());
        if (c == EOF) return true;
        std::ungetc(c, fp());
        return false;
    }
    QString readLine() {
        std::string line;
        if (fp() == nullptr) return QString();
        int c;
        while ((c = std::fgetc(fp())) != EOF && c != '\n') line += (char)c;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        return QString(line);
    }
    QTextStream& operator<<(const char* s) { if (fp()) std::fputs(s, fp()); return *this; }
    QTextStream& operator<<(const QString& s) { return *this << s.str().c_str(); }
    QTextStream& operator<<(char c) { if (fp()) std::fputc(c, fp()); return *this; }
    QTextStream& operator<<(QChar c) { return *this << c.toLatin1(); }
    QTextStream& operator<<(double v) {
        // Qt's default: 'g' with 6 significant digits
        char spec[16], buf[64];
        const char conv = nota_ == ScientificNotation ? 'e' : nota_ == FixedNotation ? 'f' : 'g';
        std::snprintf(spec, sizeof(spec), "%%%s.%d%c", (flags_ & ForceSign) ? "+" : "", prec_, conv);
        std::snprintf(buf, sizeof(buf), spec, v);
        return *this << buf;
    }
    QTextStream& operator<<(float v) { return *this << (double)v; }
    template <class I>
    typename std::enable_if<std::is_integral<I>::value && !std::is_same<I, char>::value,
                            QTextStream&>::type
    operator<<(I v) {
        char b[32];
        if (std::is_signed<I>::value)
            std::snprintf(b, sizeof(b), (flags_ & ForceSign) ? "%+lld" : "%lld", (long long)v);
        else
            std::snprintf(b, sizeof(b), (flags_ & ForceSign) ? "+%llu" : "%llu",
                          (unsigned long long)v);
        return *this << b;
    }
private:
    std::FILE* fp() { return file_ ? file_->handle() : nullptr; }
    QFile* file_ = nullptr;
    int prec_ = 6;
    RealNumberNotation nota_ = SmartNotation;
    int flags_ = 0;
};

inline void QDir::mkdir_one(const std::string& d) { ::mkdir(d.c_str(), 0777); }
