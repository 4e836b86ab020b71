// Header-only stand-in for the handful of Qt 5 classes that the reference's
// ptnee sources name (QImage, QColor, QString, QDebug, QTime, QTimer,
// QEventLoop, QMutex, QObject). Qt is not installed on this machine; the
// oracle build uses these so the reference's own .cpp files compile
// unmodified. Test infrastructure only: nothing in the product includes it.
//
// Real Qt 5 container headers include <stdlib.h>, which in C++ brings
// std::abs(float) into the global namespace; this stub does the same so that
// `abs(x)` on floats in the reference's renderer code resolves as it does in
// a Qt build.
#pragma once
#include <cstdlib>
using std::abs;
#include <chrono>
#include <cstdint>
#include <functional>
#include <iostream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

typedef unsigned int QRgb;
inline QRgb qRgb(int r, int g, int b) {
    return 0xff000000u | ((unsigned)(r & 0xff) << 16) | ((unsigned)(g & 0xff) << 8) | (unsigned)(b & 0xff);
}

namespace Qt { enum GlobalColor { black = 2, white = 3 }; }

class QString {
public:
    std::string s;
    QString() = default;
    QString(const char* c) : s(c) {}
    static QString fromStdString(const std::string& x) { QString q; q.s = x; return q; }
    QString& replace(const char* a, const char* b) {
        std::string from(a), to(b);
        size_t p = 0;
        while (!from.empty() && (p = s.find(from, p)) != std::string::npos) { s.replace(p, from.size(), to); p += to.size(); }
        return *this;
    }
    std::string toStdString() const { return s; }
};

class QSize {
public:
    int w, h;
    QSize(int w_, int h_) : w(w_), h(h_) {}
};

class QColor {
public:
    double r = 0, g = 0, b = 0;
    double redF() const { return r; }
    double greenF() const { return g; }
    double blueF() const { return b; }
};

// RGB888 image held in memory. Loading image files is not supported (no
// codec): a QImage built from a file name is empty.
class QImage {
public:
    enum Format { Format_Invalid = 0, Format_RGB888 = 13, Format_RGBA8888 = 17 };
    int w = 0, h = 0;
    std::vector<QRgb> px;
    QImage() = default;
    QImage(const QSize& s, Format) : w(s.w), h(s.h), px((size_t)s.w * s.h, 0xff000000u) {}
    explicit QImage(const QString&) {}
    QImage convertToFormat(Format) const { return *this; }
    int width() const { return w; }
    int height() const { return h; }
    void fill(Qt::GlobalColor c) { for (auto& p : px) p = (c == Qt::white) ? 0xffffffffu : 0xff000000u; }
    void setPixel(int x, int y, QRgb v) { if (x >= 0 && y >= 0 && x < w && y < h) px[(size_t)y * w + x] = v; }
    QRgb pixel(int x, int y) const { return px[(size_t)y * w + x]; }
    QColor pixelColor(int x, int y) const {
        QRgb v = pixel(x, y); QColor c;
        c.r = ((v >> 16) & 0xff) / 255.0; c.g = ((v >> 8) & 0xff) / 255.0; c.b = (v & 0xff) / 255.0;
        return c;
    }
    bool save(const QString&) const { return false; }
};

class QDebugStub {
public:
    template <class T> QDebugStub& operator<<(const T&) { return *this; }
};
inline QDebugStub qDebug() { return QDebugStub(); }

class QTime {
    std::chrono::steady_clock::time_point t0;
public:
    void start() { t0 = std::chrono::steady_clock::now(); }
    int elapsed() const {
        return (int)std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
    }
};

class QMutex {
    std::mutex m;
public:
    void lock() { m.lock(); }
    void unlock() { m.unlock(); }
    bool tryLock() { return m.try_lock(); }
};

class QObject {
public:
    template <class A, class B, class F> static void connect(A*, B, F) {}
};

class QTimer : public QObject {
public:
    int ms = 0;
    void setInterval(int v) { ms = v; }
    void start() {}
    void timeout() {}
};

// The reference polls its worker threads every 100 ms through a Qt event
// loop; here exec() just sleeps for that interval.
class QEventLoop {
public:
    int exec() { std::this_thread::sleep_for(std::chrono::milliseconds(100)); return 0; }
    void quit() {}
};
