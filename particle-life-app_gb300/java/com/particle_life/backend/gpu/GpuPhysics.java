// GpuPhysics.java — the Java 21 (Panama FFM) binding of libplgpu.so for the
// reference app: a Physics subclass whose update() runs the GPU step
// (include/plgpu.h).  It goes in backend/gpu/ beside backend/Physics.java
// and compiles with --enable-preview --release 21 (FFM is final from JDK 22
// on).  The build of this repository does not compile it (it has no Java
// toolchain); the C ABI it binds is tested through the Python binding.
package com.particle_life.backend.gpu;

import com.particle_life.backend.*;
import java.lang.foreign.*;
import java.lang.invoke.MethodHandle;
import java.nio.file.Path;
import static java.lang.foreign.ValueLayout.*;

/** Physics whose update() runs on the GPU through libplgpu.so. */
public class GpuPhysics extends Physics {
    private static final Linker LINKER = Linker.nativeLinker();
    private static final SymbolLookup LIB =
            SymbolLookup.libraryLookup(Path.of(System.getProperty("plgpu.lib", "libplgpu.so")), Arena.global());
    private static MethodHandle h(String name, FunctionDescriptor fd) {
        return LINKER.downcallHandle(LIB.find(name).orElseThrow(), fd);
    }
    // struct plg_settings { double rmax, friction, force, dt, beta; int32 wrap, accel_kind; }
    static final StructLayout SETTINGS = MemoryLayout.structLayout(
            JAVA_DOUBLE.withName("rmax"), JAVA_DOUBLE.withName("friction"), JAVA_DOUBLE.withName("force"),
            JAVA_DOUBLE.withName("dt"), JAVA_DOUBLE.withName("beta"),
            JAVA_INT.withName("wrap"), JAVA_INT.withName("accel_kind"));
    static final MethodHandle CREATE = h("plg_create", FunctionDescriptor.of(JAVA_INT, JAVA_INT, JAVA_LONG, ADDRESS));
    static final MethodHandle DESTROY = h("plg_destroy", FunctionDescriptor.of(JAVA_INT, ADDRESS));
    static final MethodHandle SET_SETTINGS = h("plg_set_settings", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS));
    static final MethodHandle SET_MATRIX = h("plg_set_matrix", FunctionDescriptor.of(JAVA_INT, ADDRESS, JAVA_INT, ADDRESS));
    static final MethodHandle UPLOAD = h("plg_upload",
            FunctionDescriptor.of(JAVA_INT, ADDRESS, JAVA_LONG, ADDRESS, ADDRESS, ADDRESS));
    static final MethodHandle STEP = h("plg_step", FunctionDescriptor.of(JAVA_INT, ADDRESS, JAVA_INT));
    static final MethodHandle DOWNLOAD = h("plg_download",
            FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS, ADDRESS, ADDRESS, ADDRESS));
    static final MethodHandle STEP_DOWNLOAD = h("plg_step_download",
            FunctionDescriptor.of(JAVA_INT, ADDRESS, JAVA_INT, ADDRESS, ADDRESS, ADDRESS, ADDRESS));
    static final MethodHandle STOP = h("plg_request_stop", FunctionDescriptor.of(JAVA_INT, ADDRESS));
    static final MethodHandle LAST_ERROR = h("plg_last_error", FunctionDescriptor.of(ADDRESS, ADDRESS));

    private final Arena arena = Arena.ofShared();
    private MemorySegment ctx = MemorySegment.NULL;
    private long capacity;
    public final double beta;

    public GpuPhysics(double beta, PositionSetter ps, MatrixGenerator mg, TypeSetter ts) {
        super((a, pos) -> { throw new UnsupportedOperationException("runs on the GPU"); }, ps, mg, ts);
        this.beta = beta;
    }

    private void check(int status, String what) {
        if (status != 0) {
            String msg = ctx.equals(MemorySegment.NULL) ? ""
                    : ((MemorySegment) invoke(LAST_ERROR, ctx)).reinterpret(4096).getString(0);
            throw new IllegalStateException(what + " failed (" + status + "): " + msg);
        }
    }

    @Override
    public void update() {
        int n = particles.length;
        if (ctx.equals(MemorySegment.NULL) || n > capacity) {
            if (!ctx.equals(MemorySegment.NULL)) invoke(DESTROY, ctx);
            MemorySegment out = arena.allocate(ADDRESS);
            capacity = Math.max(n, 1);
            check((int) invoke(CREATE, 2, capacity, out), "plg_create");
            ctx = out.get(ADDRESS, 0);
        }
        try (Arena call = Arena.ofConfined()) {
            MemorySegment s = call.allocate(SETTINGS);
            s.set(JAVA_DOUBLE, 0, settings.rmax);
            s.set(JAVA_DOUBLE, 8, settings.friction);
            s.set(JAVA_DOUBLE, 16, settings.force);
            s.set(JAVA_DOUBLE, 24, settings.dt);
            s.set(JAVA_DOUBLE, 32, beta);
            s.set(JAVA_INT, 40, settings.wrap ? 1 : 0);
            s.set(JAVA_INT, 44, 1 /* PLG_ACCEL_PARTICLE_LIFE */);
            check((int) invoke(SET_SETTINGS, ctx, s), "plg_set_settings");
            int t = settings.matrix.size();
            MemorySegment m = call.allocate(JAVA_DOUBLE, (long) t * t);
            for (int i = 0; i < t; i++)
                for (int j = 0; j < t; j++) m.setAtIndex(JAVA_DOUBLE, (long) i * t + j, settings.matrix.get(i, j));
            check((int) invoke(SET_MATRIX, ctx, t, m), "plg_set_matrix");
            // Upload: the snapshot layout of app/PhysicsSnapshot.java:50-58.
            MemorySegment pos = call.allocate(JAVA_DOUBLE, 3L * n), vel = call.allocate(JAVA_DOUBLE, 3L * n);
            MemorySegment type = call.allocate(JAVA_INT, n), id = call.allocate(JAVA_INT, n);
            for (int i = 0; i < n; i++) {
                Particle p = particles[i];
                pos.setAtIndex(JAVA_DOUBLE, 3L * i, p.position.x);
                pos.setAtIndex(JAVA_DOUBLE, 3L * i + 1, p.position.y);
                pos.setAtIndex(JAVA_DOUBLE, 3L * i + 2, p.position.z);
                vel.setAtIndex(JAVA_DOUBLE, 3L * i, p.velocity.x);
                vel.setAtIndex(JAVA_DOUBLE, 3L * i + 1, p.velocity.y);
                vel.setAtIndex(JAVA_DOUBLE, 3L * i + 2, p.velocity.z);
                type.setAtIndex(JAVA_INT, i, p.type);
            }
            check((int) invoke(UPLOAD, ctx, (long) n, pos, vel, type), "plg_upload");
            // One step whose force kernel writes the snapshot (same bits as
            // plg_step followed by plg_download).
            check((int) invoke(STEP_DOWNLOAD, ctx, 1, pos, vel, type, id), "plg_step_download");
            // Reproduce the reference's permutation of `particles`.
            Particle[] sorted = new Particle[n];
            for (int i = 0; i < n; i++) {
                Particle p = particles[id.getAtIndex(JAVA_INT, i)];
                p.position.set(pos.getAtIndex(JAVA_DOUBLE, 3L * i), pos.getAtIndex(JAVA_DOUBLE, 3L * i + 1),
                        pos.getAtIndex(JAVA_DOUBLE, 3L * i + 2));
                p.velocity.set(vel.getAtIndex(JAVA_DOUBLE, 3L * i), vel.getAtIndex(JAVA_DOUBLE, 3L * i + 1),
                        vel.getAtIndex(JAVA_DOUBLE, 3L * i + 2));
                sorted[i] = p;
            }
            particles = sorted;
        }
    }

    @Override
    public void forceUpdateStop() {
        if (!ctx.equals(MemorySegment.NULL)) invoke(STOP, ctx);
    }

    private static Object invoke(MethodHandle mh, Object... args) {
        try {
            return mh.invokeWithArguments(args);
        } catch (Throwable t) {
            throw new RuntimeException(t);
        }
    }

    private static final StructLayout RENDER_PARAMS = MemoryLayout.structLayout(
            JAVA_INT.withName("width"), JAVA_INT.withName("height"),
            JAVA_DOUBLE.withName("cam_x"), JAVA_DOUBLE.withName("cam_y"),
            JAVA_DOUBLE.withName("cam_w"), JAVA_DOUBLE.withName("cam_h"),
            JAVA_DOUBLE.withName("top_left_x"), JAVA_DOUBLE.withName("top_left_y"),
            JAVA_DOUBLE.withName("size"), JAVA_INT.withName("wrap"), JAVA_INT.withName("reserved"));
    private static final MethodHandle RENDER =
            h("plg_render", FunctionDescriptor.of(JAVA_INT, ADDRESS, ADDRESS, JAVA_INT, ADDRESS, ADDRESS));

    /** The 256 x 256 thumbnail as ARGB ints (BufferedImage.TYPE_INT_ARGB rows);
     *  palette: com.particle_life.app.color.Color per type. */
    public int[] thumbnail(com.particle_life.app.color.Color[] palette) {
        try (Arena arena = Arena.ofConfined()) {
            MemorySegment rp = arena.allocate(RENDER_PARAMS);
            rp.set(JAVA_INT, 0, 256);
            rp.set(JAVA_INT, 4, 256);
            double[] d = {0.5, 0.5, 1.0, 1.0, 0.0, 0.0, 0.015};
            for (int k = 0; k < d.length; k++) rp.set(JAVA_DOUBLE, 8 + 8L * k, d[k]);
            rp.set(JAVA_INT, 64, 0);
            MemorySegment pal = arena.allocate(JAVA_FLOAT, 4L * palette.length);
            for (int k = 0; k < palette.length; k++) {
                pal.setAtIndex(JAVA_FLOAT, 4L * k, palette[k].r);
                pal.setAtIndex(JAVA_FLOAT, 4L * k + 1, palette[k].g);
                pal.setAtIndex(JAVA_FLOAT, 4L * k + 2, palette[k].b);
                pal.setAtIndex(JAVA_FLOAT, 4L * k + 3, palette[k].a);
            }
            MemorySegment out = arena.allocate(4L * 256 * 256);
            check((int) invoke(RENDER, ctx, rp, palette.length, pal, out), "plg_render");
            int[] argb = new int[256 * 256];
            for (int i = 0; i < argb.length; i++) {
                int r = out.get(JAVA_BYTE, 4L * i) & 255, g = out.get(JAVA_BYTE, 4L * i + 1) & 255;
                int b = out.get(JAVA_BYTE, 4L * i + 2) & 255, a = out.get(JAVA_BYTE, 4L * i + 3) & 255;
                argb[i] = a << 24 | r << 16 | g << 8 | b;
            }
            return argb;
        }
    }
}
