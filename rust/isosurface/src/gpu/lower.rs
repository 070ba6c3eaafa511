//! Lowering of the crate's sources to the library's device program (the
//! "Source programs" format of include/isosurface_gpu.h): ops in postfix
//! order over a value stack, each with an index into one f32 constant pool.
//!
//! Not compiled here (no Rust toolchain on the machines this library was
//! built on); it mirrors isosurface_gb300/source.py, whose programs the
//! library's tests check against the oracle bit for bit.

use crate::{
    implicit::{Cylinder, Difference, Intersection, RectangularPrism, Sphere, Torus, Union},
    sampler::Sampler,
    source::{CentralDifference, ScalarSource},
};

const MAGIC: u32 = 0x314F_5349; // "ISO1"

const OP_SPHERE: u32 = 0x10;
const OP_BOX: u32 = 0x11;
const OP_CYLINDER: u32 = 0x12;
const OP_TORUS: u32 = 0x13;
const OP_UNION: u32 = 0x20;
const OP_INTERSECTION: u32 = 0x21;
const OP_DIFFERENCE: u32 = 0x22;
const OP_CD_BEGIN: u32 = 0x40;
const OP_CD_END: u32 = 0x41;

/// Ops and constants of a program being built.
#[derive(Default)]
pub struct ProgramBuilder {
    ops: Vec<u32>,
    consts: Vec<f32>,
}

impl ProgramBuilder {
    /// Appends constants and returns the index of the first one.
    pub fn constants(&mut self, values: &[f32]) -> u32 {
        let at = self.consts.len() as u32;
        assert!(at < (1 << 24), "program has too many constants");
        self.consts.extend_from_slice(values);
        at
    }

    /// Appends one op whose argument is a constant index.
    pub fn op(&mut self, code: u32, arg: u32) {
        self.ops.push((arg << 8) | code);
    }

    /// The program bytes: a 16-byte header, the ops, the constants (all
    /// little-endian).
    pub fn bytes(&self) -> Vec<u8> {
        let mut out = Vec::with_capacity(16 + 4 * (self.ops.len() + self.consts.len()));
        for w in [MAGIC, self.ops.len() as u32, self.consts.len() as u32, 0] {
            out.extend_from_slice(&w.to_le_bytes());
        }
        for op in &self.ops {
            out.extend_from_slice(&op.to_le_bytes());
        }
        for c in &self.consts {
            out.extend_from_slice(&c.to_le_bytes());
        }
        out
    }
}

/// A source the GPU library can evaluate: it appends its own ops.  The
/// library has no CPU fallback, so an `extract` on the GPU path requires this
/// bound on its source in addition to the reference's `Sample` bounds.
pub trait LowerToDevice {
    fn lower(&self, program: &mut ProgramBuilder);

    /// The whole program of this source.
    fn program_bytes(&self) -> Vec<u8> {
        let mut b = ProgramBuilder::default();
        self.lower(&mut b);
        b.bytes()
    }
}

impl LowerToDevice for Sphere {
    fn lower(&self, p: &mut ProgramBuilder) {
        let at = p.constants(&[self.radius]);
        p.op(OP_SPHERE, at);
    }
}

impl LowerToDevice for RectangularPrism {
    fn lower(&self, p: &mut ProgramBuilder) {
        let h = self.half_extent;
        let at = p.constants(&[h.x, h.y, h.z]);
        p.op(OP_BOX, at);
    }
}

impl LowerToDevice for Cylinder {
    fn lower(&self, p: &mut ProgramBuilder) {
        let at = p.constants(&[self.radius, self.half_length]);
        p.op(OP_CYLINDER, at);
    }
}

impl LowerToDevice for Torus {
    fn lower(&self, p: &mut ProgramBuilder) {
        let at = p.constants(&[self.radius, self.tube_radius]);
        p.op(OP_TORUS, at);
    }
}

/// min(a, b) (csg.rs Union).
impl<A: LowerToDevice, B: LowerToDevice> LowerToDevice for Union<A, B> {
    fn lower(&self, p: &mut ProgramBuilder) {
        self.a.lower(p);
        self.b.lower(p);
        p.op(OP_UNION, 0);
    }
}

/// max(a, b) (csg.rs Intersection).
impl<A: LowerToDevice, B: LowerToDevice> LowerToDevice for Intersection<A, B> {
    fn lower(&self, p: &mut ProgramBuilder) {
        self.a.lower(p);
        self.b.lower(p);
        p.op(OP_INTERSECTION, 0);
    }
}

/// max(b, -a): b minus a (csg.rs Difference).
impl<A: LowerToDevice, B: LowerToDevice> LowerToDevice for Difference<A, B> {
    fn lower(&self, p: &mut ProgramBuilder) {
        self.a.lower(p);
        self.b.lower(p);
        p.op(OP_DIFFERENCE, 0);
    }
}

/// Normals of the wrapped source by central differences (source.rs).  The
/// epsilon field is private to the crate, which is why this module lives in
/// the crate rather than beside it.
impl<S: ScalarSource + LowerToDevice> LowerToDevice for CentralDifference<S> {
    fn lower(&self, p: &mut ProgramBuilder) {
        let at = p.constants(&[self.epsilon]);
        p.op(OP_CD_BEGIN, at);
        self.source.lower(p);
        p.op(OP_CD_END, 0);
    }
}

/// A Sampler only borrows its source (sampler.rs).
impl<'a, S: LowerToDevice> LowerToDevice for Sampler<'a, S> {
    fn lower(&self, p: &mut ProgramBuilder) {
        self.source.lower(p);
    }
}
