"""moldyn-cli drop-in: the reference's command line (cli/src/args.rs:5-176,
cli/src/commands.rs) with the force / integration path on the GPU.

    python -m moldyn_gb300 -f DIR [--time] [--frames-per-save N] COMMAND ...

Commands and flags are the reference's: generate-default-potentials,
set-potential, initialize, solve, solve-macro-parameters, check-impulse,
particle-count, generate-velocities-histogram.  Engine options are extra
flags of `solve` / `solve-macro-parameters` (--precision, --reference-order,
--skin).  Differences from the reference, on purpose:
  * --frames-per-save is honoured (the reference parses it and ignores it):
    frame files are written every N steps, numbered by step as before.
  * initialize takes --seed (the reference's velocity draw is unseeded).
  * unimplemented choices (custom integrator/thermostat/barostat/potential)
    exit with an error message instead of panicking.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

from . import io as mio
from .core import K_B, ParticleDatabase, State


def _fail(msg: str):
    print(f"error: {msg}", file=sys.stderr)
    sys.exit(2)


def _parser():
    ap = argparse.ArgumentParser(prog="moldyn-cli")
    ap.add_argument("-f", "--file", required=True, help="path to the simulation directory")
    ap.add_argument("--time", action="store_true", help="measure time of work")
    ap.add_argument("--frames-per-save", type=int, default=1, help="how often to save state")
    sub = ap.add_subparsers(dest="command", required=True)

    sub.add_parser("generate-default-potentials")
    sp = sub.add_parser("set-potential")
    sp.add_argument("-i", "--particle-types", type=int, nargs=2, required=True)
    sp.add_argument("-p", "--potential", choices=["lennard-jones", "custom"], required=True)
    sp.add_argument("--params", type=float, nargs="+", required=True)

    ini = sub.add_parser("initialize")
    ini.add_argument("-t", "--crystal-cell-type", choices=["u", "fcc"], required=True)
    ini.add_argument("-s", "--size", type=int, nargs=3, required=True)
    ini.add_argument("-n", "--particle-name", required=True)
    ini.add_argument("-m", "--particle-mass", type=float, required=True)
    ini.add_argument("-r", "--particle-radius", type=float, required=True)
    ini.add_argument("-l", "--lattice-cell", type=float, required=True)
    ini.add_argument("-T", "--temperature", type=float, required=True)
    ini.add_argument("--seed", type=int, default=0)

    so = sub.add_parser("solve")
    so.add_argument("--threads-count", type=int, default=None, help="accepted; the GPU ignores it")
    so.add_argument("-s", "--state-number", type=int, required=True)
    so.add_argument("-i", "--integrate-method", choices=["verlet-method", "custom"], required=True)
    so.add_argument("--custom-method", default=None)
    so.add_argument("--barostat", choices=["berendsen", "custom"], default=None)
    so.add_argument("--barostat-params", type=float, nargs="+", default=None)
    so.add_argument("-P", "--pressure", type=float, default=None)
    so.add_argument("--thermostat", choices=["berendsen", "nose-hoover", "custom"], default=None)
    so.add_argument("--thermostat-params", type=float, nargs="+", default=None)
    so.add_argument("-T", "--temperature", type=float, default=None)
    so.add_argument("-p", "--use-potentials", action="store_true")
    so.add_argument("-c", "--iteration-count", type=int, required=True)
    so.add_argument("-t", "--delta-time", type=float, required=True)
    _engine_flags(so)

    sm = sub.add_parser("solve-macro-parameters")
    for short, name in (("-k", "kinetic-energy"), ("-p", "potential-energy"), ("-t", "thermal-energy"),
                        ("-T", "temperature"), ("-P", "pressure"), ("-c", "custom")):
        sm.add_argument(short, f"--{name}", action="store_true")
    sm.add_argument("-C", "--custom-name", default=None)
    sm.add_argument("-A", "--all", action="store_true")
    sm.add_argument("--use-potentials", action="store_true")
    _engine_flags(sm)

    sub.add_parser("check-impulse")
    sub.add_parser("particle-count")
    hg = sub.add_parser("generate-velocities-histogram")
    hg.add_argument("-s", "--state-number", type=int, required=True)
    hg.add_argument("--particle-types", type=int, nargs="+", required=True)
    rd = sub.add_parser("render", help="headless picture of a saved frame (the GUI viewer's shading)")
    rd.add_argument("-s", "--state-number", type=int, default=0)
    rd.add_argument("-o", "--out", required=True, help="output image (binary PPM)")
    rd.add_argument("--width", type=int, default=1920)
    rd.add_argument("--height", type=int, default=1080)
    rd.add_argument("--color-by", choices=["type", "speed"], default="type")
    rd.add_argument("--speed-range", type=float, nargs=2, default=[0.0, 1.0])
    rd.add_argument("--eye", type=float, nargs=3, default=None, help="camera position (default: frames the box)")
    rd.add_argument("--forward", type=float, nargs=3, default=[1.0, 0.0, 0.0])
    rd.add_argument("--fovy", type=float, default=70.0)
    rd.add_argument("--no-box", action="store_true")
    return ap


def _engine_flags(p):
    p.add_argument("--precision", choices=["fp64", "mixed"], default="fp64",
                   help="fp64 (default): the reference's arithmetic; mixed: FP32 pair maths")
    p.add_argument("--reference-order", choices=["on", "off"], default="on",
                   help="fp64 only: reproduce the reference's summation order (bit-identical results)")
    p.add_argument("--skin", type=float, default=0.0, help="Verlet skin (0: 0.3 sigma)")


def _make_engine(args):
    from .engine import Engine
    ref = args.precision == "fp64" and args.reference_order == "on"
    return Engine(precision=args.precision, reference_order=ref, skin=args.skin)


def _potentials(directory, use):
    from .solver import PotentialsDatabase
    pdb = PotentialsDatabase()
    if use:
        pdb.load_potentials_from_file(directory)
    return pdb


def _bind(eng, pdb, state: State):
    ntypes = state.ntypes
    for a in range(ntypes):
        for b in range(a, ntypes):
            p = pdb.get_potential(a, b)
            eng.set_potential_raw(a, b, p.sigma, p.eps, p.r_cut, p.u_cut)
    eng.upload(state.ids, state.positions, state.velocities, state.masses_per_type(), state.boundary_box)


# ---------------------------------------------------------------------------
def cmd_generate_default_potentials(args):
    """commands.rs:198-202."""
    from .solver import Potential, PotentialsDatabase
    pdb = PotentialsDatabase()
    pdb.set_potential(0, 0, Potential.new_lennard_jones(0.3418, 1.712))
    pdb.save_potentials_to_file(args.file)


def cmd_set_potential(args):
    """commands.rs:204-217: load potentials.json, set the pair, save."""
    from .solver import Potential, PotentialsDatabase
    if args.potential == "custom":
        _fail("custom potentials are not implemented (todo!() in the reference)")
    if not os.path.exists(os.path.join(args.file, "potentials.json")):
        _fail("Can't open file: potentials.json (run generate-default-potentials first)")
    pdb = PotentialsDatabase()
    pdb.load_potentials_from_file(args.file)
    pdb.set_potential(args.particle_types[0], args.particle_types[1],
                      Potential.new_lennard_jones(args.params[0], args.params[1]))
    pdb.save_potentials_to_file(args.file)


def cmd_initialize(args):
    """commands.rs:219-256."""
    from .initializer import UnitCell, lattice_positions, maxwell_boltzmann
    ParticleDatabase.add(0, args.particle_name, args.particle_mass, args.particle_radius)
    cell = UnitCell.U if args.crystal_cell_type == "u" else UnitCell.FCC
    pos = lattice_positions(cell, args.size, args.lattice_cell)
    box = np.array([args.lattice_cell * s for s in args.size], dtype=np.float64)
    vel = maxwell_boltzmann(len(pos), args.temperature, args.particle_mass, args.seed)
    st = State(pos, vel, np.zeros(len(pos), dtype=np.uint16), box)
    mio.save_state(args.file, 0, st)
    ParticleDatabase.save_particles_data(args.file)


def cmd_solve(args):
    """commands.rs:258-367 (the state is device resident between saved frames)."""
    from .initializer import Barostat, Thermostat
    if args.integrate_method != "verlet-method":
        _fail("custom integrators are not implemented (todo!() in the reference)")
    mio.load_particles(args.file)
    state = mio.load_state(args.file, args.state_number)
    pdb = _potentials(args.file, args.use_potentials)
    th = ba = None
    t0 = p0 = 0.0
    if args.thermostat is not None:
        if args.thermostat == "custom":
            _fail("custom thermostats are not implemented (todo!() in the reference)")
        name = "Berendsen" if args.thermostat == "berendsen" else "Nose-Hoover"
        if not args.thermostat_params:
            _fail(f"No thermostat parameters. Need tau for {name}")
        if args.temperature is None:
            _fail("No temperature was passed")
        th = (Thermostat.Berendsen(args.thermostat_params[0]) if args.thermostat == "berendsen"
              else Thermostat.NoseHoover(args.thermostat_params[0]))
        t0 = args.temperature
    if args.barostat is not None:
        if args.barostat != "berendsen":
            _fail("custom barostats are not implemented (todo!() in the reference)")
        if not args.barostat_params or len(args.barostat_params) < 2:
            _fail("No barostat parameters. Need beta and tau for Berendsen")
        if args.pressure is None:
            _fail("No pressure was passed")
        ba, p0 = Barostat.Berendsen(args.barostat_params[0], args.barostat_params[1]), args.pressure
    eng = _make_engine(args)
    _bind(eng, pdb, state)
    eng.compute_forces()                                       # commands.rs:278
    boxes = mio.load_boxes(args.file)
    fps = max(1, args.frames_per_save)
    order = np.argsort(state.ids, kind="stable")
    ids = state.ids[order]
    done = 0
    # frames are formatted and written on a background thread while the
    # device runs the next steps
    with mio.FrameWriter(args.file) as writer:
        while done < args.iteration_count:
            if done % fps == 0:
                out = eng.download()
                frame = args.state_number + done
                if len(boxes) > frame:
                    boxes[frame] = out["box"]
                else:
                    while len(boxes) < frame:
                        boxes.append(out["box"])
                    boxes.append(out["box"])
                writer.submit(frame, ids, out["pos"][order], out["vel"][order])
            n = min(fps - done % fps, args.iteration_count - done)
            eng.step(n, args.delta_time, thermostat=th, target_temperature=t0, barostat=ba, target_pressure=p0)
            done += n
        out = eng.download()
        frame = args.state_number + args.iteration_count
        while len(boxes) < frame:
            boxes.append(out["box"])
        if len(boxes) > frame:
            boxes[frame] = out["box"]
        else:
            boxes.append(out["box"])
        writer.submit(frame, ids, out["pos"][order], out["vel"][order])
    mio.save_boxes(args.file, boxes)
    eng.close()


def cmd_solve_macro(args):
    """commands.rs:380-450: recompute forces for every frame, then the macro
    parameters of type 0 (temperature with the count of all particles)."""
    if args.all:
        args.kinetic_energy = args.potential_energy = args.thermal_energy = True
        args.temperature = args.pressure = True
    if args.custom:
        _fail("custom macro parameters are not implemented (todo!() in the reference)")
    mio.load_particles(args.file)
    pdb = _potentials(args.file, args.use_potentials)
    eng = _make_engine(args)
    rows = []
    for i in mio.frame_numbers(args.file):
        state = mio.load_state(args.file, i)
        _bind(eng, pdb, state)
        eng.compute_forces()
        m = eng.macro(0)
        count = state.n
        row = {k: 0.0 for k in mio.MACRO_HEADER}
        row["iteration"] = i
        if args.kinetic_energy:
            row["kinetic_energy"] = m["kinetic_energy"]
            row["unit_kinetic_energy"] = m["kinetic_energy"] / count
        if args.potential_energy:
            row["potential_energy"] = m["potential_energy"]
            row["unit_potential_energy"] = m["potential_energy"] / count
        if args.thermal_energy or args.temperature:
            row["thermal_energy"] = m["thermal_energy"]
            row["unit_thermal_energy"] = m["thermal_energy"] / count
        if args.temperature:
            row["temperature"] = (2.0 * m["thermal_energy"]) / (3.0 * float(count) * K_B) * 100.0
        if args.pressure:
            row["pressure"] = m["pressure"]
        rows.append(row)
    mio.save_macro(args.file, rows)
    eng.close()


def cmd_check_impulse(args):
    """commands.rs:452-478 (momentum from the frame files, host arithmetic)."""
    mio.load_particles(args.file)
    frames = mio.frame_numbers(args.file)
    for label, f in (("First frame", frames[0]), ("Last frame", frames[-1])):
        print(label)
        st = mio.load_state(args.file, f)
        for t in range(st.ntypes):
            m = ParticleDatabase.get_particle_mass(t)
            p = np.zeros(3)
            for v in st.velocities[st.ids == t]:
                p += v * m
            print(f"type = {t};|p| = {np.sqrt(p @ p):.15f};p = [{p[0]:.15f}, {p[1]:.15f}, {p[2]:.15f}]")


def cmd_particle_count(args):
    mio.load_particles(args.file)
    st = mio.load_state(args.file, 0)
    print(f"Particle count: {st.n}")


def cmd_histogram(args):
    """commands.rs:490-515: hist.csv with x,y,z velocity rows."""
    mio.load_particles(args.file)
    st = mio.load_state(args.file, args.state_number)
    with open(os.path.join(args.file, "hist.csv"), "w", newline="") as f:
        f.write("x,y,z\n")
        for t in args.particle_types:
            for v in st.velocities[st.ids == t]:
                f.write(",".join(mio.fmt_float(c) for c in v) + "\n")


def cmd_render(args):
    """The GUI viewer's picture of one frame (gui/src/visualizer/window.rs:940-990),
    rendered on the GPU without a window and written as a PPM image."""
    from . import render as rnd
    mio.load_particles(args.file)
    st = mio.load_state(args.file, args.state_number)
    if args.eye is None:
        cam = rnd.framing_camera(st.boundary_box, args.width, args.height, args.fovy)
        cam.update(cam.eye, args.forward, args.width, args.height)
    else:
        cam = rnd.Camera(args.eye, args.fovy, args.width, args.height, args.forward)
    mode = rnd.MODE_TYPE if args.color_by == "type" else rnd.MODE_SPEED
    img = rnd.render_state(st, cam, args.width, args.height, mode, speed_range=args.speed_range,
                           draw_box=not args.no_box)
    rnd.write_ppm(args.out, img)


COMMANDS = {"generate-default-potentials": cmd_generate_default_potentials, "set-potential": cmd_set_potential,
            "initialize": cmd_initialize, "solve": cmd_solve, "solve-macro-parameters": cmd_solve_macro,
            "check-impulse": cmd_check_impulse, "particle-count": cmd_particle_count,
            "generate-velocities-histogram": cmd_histogram, "render": cmd_render}


def main(argv=None):
    args = _parser().parse_args(argv)
    start = time.perf_counter()
    COMMANDS[args.command](args)
    if args.time:
        print(f"Time elapsed: {time.perf_counter() - start}")


if __name__ == "__main__":
    main()
